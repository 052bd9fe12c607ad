"""Volume sampling (fl_sample_volume, the reference's sampleParticles) and
the brick writer, against the oracle's C restatement of the kernel."""
from __future__ import annotations

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import scenes
from fluids3_gb300.volume import brick_box, read_bricks, save_bricks
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-5     # the sums differ only through CUDA's and libm's expf


def _state(s):
    """Sorted positions and the grid (C cells) after the sampler's sort."""
    return s.GetBuffer(F.FPOS), s.GetBuffer(F.FGRIDOFF), s.GetBuffer(F.FGRIDCNT)


def _close(got, want):
    scale = max(float(np.abs(want).max()), 1e-30)
    assert np.allclose(got, want, rtol=RTOL, atol=RTOL * scale), float(np.abs(got - want).max() / scale)


def test_sample_volume_matches_the_oracle():
    sc = scenes.dam_break(n=20000)
    p = sc.params
    with F.FluidSystem(p, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        s.RunSteps(10)
        lo, hi = np.array(p.bound_min[:], np.float32), np.array(p.bound_max[:], np.float32)
        for res in ((32, 24, 16), (7, 5, 3), (1, 1, 1)):
            got = s.SampleParticles(res, lo, hi, 0.01)
            pos, off, cnt = _state(s)
            want = O.sample_volume(p, pos, off, cnt, res, lo, hi, 0.01)
            _close(got, want)
        assert (got >= 0).all()
        # a box around the fluid with a finer lattice, and outside-grid voxels read 0
        lo2 = np.array((-40.0, -5.0, -40.0), np.float32)
        hi2 = np.array((40.0, 20.0, 40.0), np.float32)
        got = s.SampleParticles((40, 20, 40), lo2, hi2, 1.0, sort_first=False)
        want = O.sample_volume(p, pos, off, cnt, (40, 20, 40), lo2, hi2, 1.0)
        _close(got, want)
        assert got[:, :, 0].max() == 0.0 and got.max() > 0


def test_sample_volume_into_device_memory_and_errors():
    torch = pytest.importorskip("torch")
    sc = scenes.dam_break(n=5000)
    with F.FluidSystem(sc.params, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        with pytest.raises(F.FluidsError) as e:             # no grid yet and no sort asked for
            s.SampleParticles((4, 4, 4), (-30, 0, -30), (30, 60, 30), sort_first=False)
        assert e.value.code == -6
        host = s.SampleParticles((16, 16, 16), (-30, 0, -30), (30, 60, 30))
        dev = torch.empty((16, 16, 16), dtype=torch.float32, device="cuda")
        s.SampleParticles((16, 16, 16), (-30, 0, -30), (30, 60, 30), sort_first=False, out=dev.data_ptr())
        assert np.array_equal(dev.cpu().numpy(), host)
        with pytest.raises(F.FluidsError) as e:
            s.SampleParticles((0, 4, 4), (-30, 0, -30), (30, 60, 30))
        assert e.value.code == -1


def test_bricks_file(tmp_path):
    sc = scenes.dam_break(n=20000)
    p = sc.params
    with F.FluidSystem(p, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        s.RunSteps(5)
        path = tmp_path / "frame0005.bricks"
        n = save_bricks(s, path, vol_res=(64, 64, 64), brick=16, thresh=1e-6)
        bricks = read_bricks(path)
        assert n == len(bricks) and 0 < n < 64
        lo, hi = np.array(p.bound_min[:], np.float32), np.array(p.bound_max[:], np.float32)
        for origin, blo, bhi, size, data in bricks:
            assert size == (16, 16, 16)
            b = np.array(origin) // 16
            elo, ehi = brick_box(lo, hi, (64, 64, 64), b, (16, 16, 16))
            assert np.array_equal(blo, elo) and np.array_equal(bhi, ehi)
            again = s.SampleParticles(size, blo, bhi, 0.01, sort_first=False)
            assert np.array_equal(data, again)
