"""The reference's own GPU kernels against the product, on the same input.

fluids4.0/fluid_kernels.cu is built for sm_103a with its build's flags and
driven by oracle/ref_gpu.py as FluidSystem drives it (module load, launch
shapes, the RUN_GPU_FULL phase sequence). The reference ranks points in a
cell by atomics, so its within-cell order (gndx, and with it the sorted slot
of each point) varies from run to run; points are matched by a unique id in
the colour buffer, which both move with the sort.

  * integer outputs -- cells, counts, offsets, the points of every cell --
    agree exactly;
  * floats: the reference is built with --use_fast_math (FMA contraction,
    approximate square root and division) and sums each cell in its atomic
    order, while the product follows the reference source's arithmetic
    exactly as the host evaluates it. Densities agree within 1e-5
    (relative); forces computed by both from the same densities within
    1e-4 of the forces' RMS; one advance from the same forces within 2e-5
    world units (positions) and 1e-5 relative (velocities); five full Runs
    from the same start within 1e-3 world units.
"""
from __future__ import annotations

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import scenes
from oracle import ref_gpu as R

from helpers import assert_bit_equal

pytestmark = pytest.mark.gpu

if not R.available():
    pytest.skip("the reference's GPU module is not built (reference tree absent at build time)",
                allow_module_level=True)

UNDEF = 0xFFFFFFFF


@pytest.fixture(scope="module")
def scene():
    sc = scenes.dam_break()          # 32,768 points, the reference's CPU-runnable case
    ids = np.arange(sc.n, dtype=np.uint32)
    return sc, ids


def by_id(ids_per_slot, values):
    out = np.empty_like(values)
    out[ids_per_slot] = values
    return out


def test_phases_agree_with_the_reference_gpu_kernels(scene):
    sc, ids = scene
    p, n = sc.params, sc.n
    with R.RefGpu(p, n) as ref, F.FluidSystem(p, n) as s:
        ref.set_state(sc.pos, sc.vel, sc.veval, ids)
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=ids)

        # insert: the same cell for every point, the same counts; the
        # reference's ranks are some order of 0..count-1 in each cell
        ref.insert()
        r_gcell, r_gndx, r_cnt = ref.get(R.FGCELL), ref.get(R.FGNDX), ref.get(R.FGRIDCNT)
        gcell, gndx, gcnt = s.InsertParticlesCUDA(readback=True)
        assert_bit_equal(gcell, r_gcell, "insert gcell")
        assert_bit_equal(gcnt[:p.gridTotal], r_cnt, "insert gridcnt")
        inr = r_gcell != UNDEF
        assert inr.all(), "the dam break's start state lies inside the grid"
        assert (r_gndx < r_cnt[r_gcell]).all()
        key = r_gcell.astype(np.int64) * n + r_gndx
        assert np.unique(key).size == n, "two points share a (cell, rank)"

        # prefix sum: exclusive offsets, exactly
        ref.prefix_sum(1)
        r_off = ref.get(R.FGRIDOFF)
        goff = s.PrefixSumCellsCUDA(1, readback=True)
        assert_bit_equal(goff[:p.gridTotal], r_off, "gridoff")
        want = np.concatenate([[0], np.cumsum(r_cnt, dtype=np.uint64)[:-1]]).astype(np.uint32)
        assert_bit_equal(r_off, want, "reference offsets are the exclusive scan")

        # counting sort: every cell holds the same points; each point's
        # fields moved unchanged
        ref.counting_sort()
        s.CountingSortFullCUDA()
        r_ids, o_ids = ref.get(R.FCLR), s.GetBuffer(F.FCLR)
        r_slot_cell, o_slot_cell = ref.get(R.FGCELL), s.GetBuffer(F.FGCELL)
        assert np.unique(r_ids).size == n and np.unique(o_ids).size == n
        assert_bit_equal(o_slot_cell, r_slot_cell, "cell of every slot")
        assert_bit_equal(by_id(o_ids, o_slot_cell), by_id(r_ids, r_slot_cell), "cell of every point")
        for buf in (R.FPOS, R.FVEL, R.FVEVAL):
            assert_bit_equal(by_id(o_ids, s.GetBuffer(buf)), by_id(r_ids, ref.get(buf)), f"sorted buffer {buf}")
        assert_bit_equal(ref.get(R.FGRID), np.arange(n, dtype=np.uint32), "reference FGRID after a full sort")

        # density
        ref.pressure()
        s.ComputePressureCUDA()
        o_rho = by_id(o_ids, s.GetBuffer(F.FPRESS))
        r_rho = by_id(r_ids, ref.get(R.FPRESS))
        np.testing.assert_allclose(r_rho, o_rho, rtol=1e-5, atol=0)

        # force, both from the product's densities
        ref.put(R.FPRESS, o_rho[r_ids])
        ref.force()
        s.ComputeForceCUDA()
        o_f = by_id(o_ids, s.GetBuffer(F.FFORCE))
        r_f = by_id(r_ids, ref.get(R.FFORCE))
        rms = float(np.sqrt(np.mean(np.sum(o_f.astype(np.float64) ** 2, axis=1))))
        assert rms > 0
        assert np.abs(r_f - o_f).max() <= 1e-4 * rms, (np.abs(r_f - o_f).max(), rms)

        # advance, both from the product's forces
        ref.put(R.FFORCE, o_f[r_ids])
        ref.advance(0.0)
        s.AdvanceCUDA(0.0, p.dt, p.sim_scale)
        np.testing.assert_allclose(by_id(r_ids, ref.get(R.FPOS)), by_id(o_ids, s.GetBuffer(F.FPOS)),
                                   rtol=0, atol=2e-5)
        for buf in (R.FVEL, R.FVEVAL):
            o = by_id(o_ids, s.GetBuffer(buf))
            np.testing.assert_allclose(by_id(r_ids, ref.get(buf)), o, rtol=1e-5,
                                       atol=1e-5 * float(np.abs(o).max()))


def test_five_runs_agree_with_the_reference_gpu_kernels(scene):
    sc, ids = scene
    p, n = sc.params, sc.n
    with R.RefGpu(p, n) as ref, F.FluidSystem(p, n) as s:
        ref.set_state(sc.pos, sc.vel, sc.veval, ids)
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=ids)
        t = 0.0
        for _ in range(5):
            t = ref.run(t)
            s.Run()
        assert abs(s.time - t) == 0.0, "float time accumulates as the reference's AdvanceTime"
        r_ids, o_ids = ref.get(R.FCLR), s.GetBuffer(F.FCLR)
        assert np.unique(r_ids).size == n and np.unique(o_ids).size == n
        d = np.abs(by_id(r_ids, ref.get(R.FPOS)) - by_id(o_ids, s.GetBuffer(F.FPOS)))
        assert d.max() <= 1e-3, d.max()
        assert int(ref.get(R.FGRIDCNT).sum()) == n
