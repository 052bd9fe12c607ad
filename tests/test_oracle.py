"""CPU tests of the oracle: pinned against fixtures made by the reference's own
kernel source (tests/golden/make_golden.py) and, where the reference tree is
present, against that source built on the host right now."""
from __future__ import annotations

import json

import numpy as np
import pytest

from fluids3_gb300 import scenes
from oracle import oracle as O

from helpers import (FIELDS, assert_bit_equal, density_normwise_err, density_rel_err, digest,
                     force_rel_err)

UNDEF = 0xFFFFFFFF


def test_kat_insert_scan_sort(golden_dir):
    g = np.load(golden_dir / "kat_insert_64.npz")
    p = O.params_from_bytes(g["params"])
    st = O.State.new(p, g["pos"])
    O.insert(p, st)
    assert_bit_equal(st.gcell, g["gcell"], "gcell")
    assert_bit_equal(st.gndx, g["gndx"], "gndx")
    assert_bit_equal(st.cnt[:-1], g["gridcnt"], "gridcnt")
    assert st.cnt[-1] == 0
    O.prefix_sum(p, st)
    assert_bit_equal(st.off[:-1], g["gridoff"], "gridoff")
    O.counting_sort(p, st)
    assert_bit_equal(st.pos, g["sorted_pos"], "sorted pos")
    assert_bit_equal(st.gcell, g["sorted_gcell"], "sorted gcell")
    assert_bit_equal(st.gndx, g["sorted_gndx"], "sorted gndx")


def test_kat_is_hand_checkable(golden_dir):
    # 64 points dealt round-robin over 6 cells: the first four cells get 11
    # points, the last two 10, and gndx counts up in index order per cell.
    g = np.load(golden_dir / "kat_insert_64.npz")
    cnt = g["gridcnt"]
    assert sorted(cnt[cnt > 0].tolist()) == [10, 10, 11, 11, 11, 11]
    for k in range(6):
        idx = np.arange(k, 64, 6)
        assert (g["gcell"][idx] == g["gcell"][k]).all()
        assert g["gndx"][idx].tolist() == list(range(idx.size))


def test_dam_break_2000_every_phase(golden_dir):
    g = np.load(golden_dir / "dam_break_2000.npz")
    p = O.params_from_bytes(g["params"])
    st = O.State.new(p, g["in_pos"], g["in_vel"], g["in_veval"], g["in_clr"])
    O.insert(p, st)
    assert_bit_equal(st.gcell, g["ins_gcell"], "insert gcell")
    assert_bit_equal(st.gndx, g["ins_gndx"], "insert gndx")
    assert_bit_equal(st.cnt[:-1], g["ins_gridcnt"], "insert gridcnt")
    O.prefix_sum(p, st)
    assert_bit_equal(st.off[:-1], g["gridoff"], "gridoff")
    O.counting_sort(p, st)
    for k in ("pos", "vel", "veval", "clr", "gcell", "gndx"):
        assert_bit_equal(getattr(st, k), g[f"sort_{k}"], f"sorted {k}")
    O.density(p, st)
    assert_bit_equal(st.press, g["press"], "density")
    O.force(p, st)
    assert_bit_equal(st.force, g["force"], "force")
    O.advance(p, st, 0.0, p.dt, p.sim_scale)
    for k in ("pos", "vel", "veval"):
        assert_bit_equal(getattr(st, k), g[f"adv_{k}"], f"advanced {k}")


def test_dam_break_2000_rollout(golden_dir):
    g = np.load(golden_dir / "dam_break_2000.npz")
    p = O.params_from_bytes(g["params"])
    st = O.State.new(p, g["in_pos"], g["in_vel"], g["in_veval"], g["in_clr"])
    t = O.run(p, st, 20, 0.0)
    assert np.float32(t) == g["s20_time"]
    for k in FIELDS:
        assert_bit_equal(getattr(st, k), g[f"s20_{k}"], f"step-20 {k}")


@pytest.mark.parametrize("name", ["dam_break_32k", "wave_tank_60000"])
def test_rollout_digests(golden_dir, name):
    rec = json.loads((golden_dir / "digests.json").read_text())[name]
    p = O.params_from_bytes(bytes.fromhex(rec["params"]))
    sc = scenes.dam_break() if name == "dam_break_32k" else scenes.wave_tank(n=rec["n"])
    import hashlib
    assert hashlib.sha256(sc.pos.tobytes() + sc.clr.tobytes()).hexdigest() == rec["inputs"], \
        "scene generator no longer reproduces the fixture inputs"
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    t, done = 0.0, 0
    for key in sorted((k for k in rec if k.startswith("step_")), key=lambda k: int(k[5:])):
        m = int(key[5:])
        t = O.run(p, st, m - done, t, threads=4)
        done = m
        assert digest(st.__dict__) == rec[key], f"{name} diverged by step {m}"


@pytest.mark.skipif(not O.ref_available(), reason="reference tree absent: tier-1 oracle not built")
@pytest.mark.parametrize("grid_density", [0.75, 2.0, 1.2])
def test_restatement_matches_reference_source_live(grid_density):
    """Random jittered blocks at three grid densities (gridSrch 2, 3 and 2
    with a cell between h and 2h): every field bit-equal for 8 steps."""
    sc = scenes.dam_break(n=3000, seed=11)
    p = scenes.make_params((-30.0, 0.0, -30.0), (30.0, 60.0, 30.0), grid_density=grid_density,
                           bound_slope=0.05, bound_friction=0.1)
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    R = O.RefKernels(p, sc.pos, sc.vel, sc.veval, sc.clr)
    t = tr = 0.0
    for step in range(8):
        t = O.run(p, st, 1, t)
        tr = R.run(1, tr)
        assert st.cnt[-1] == 0
        for k in FIELDS:
            assert_bit_equal(getattr(st, k), R.buf[k], f"step {step} {k} (grid_density {grid_density})")
        assert_bit_equal(st.cnt[:-1], R.buf["gridcnt"], "gridcnt")
        assert_bit_equal(st.off[:-1], R.buf["gridoff"], "gridoff")


@pytest.mark.skipif(not O.ref_available(), reason="reference tree absent: tier-1 oracle not built")
def test_moving_wall_matches_reference_source_live():
    sc = scenes.wave_tank(n=20000, wall_force=0.3, wall_freq=8.0)
    p = sc.params
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    R = O.RefKernels(p, sc.pos, sc.vel, sc.veval, sc.clr)
    t = O.run(p, st, 5, 0.7)
    R.run(5, 0.7)
    for k in FIELDS:
        assert_bit_equal(getattr(st, k), R.buf[k], f"{k}")


def test_out_of_range_points_go_to_the_tail():
    """Clean semantics for points outside [1, gridScanMax]: after the sort they
    sit behind every in-range point in their original index order, with
    GRID_UNDEF cells, density 0, force 0, and advance parks them at -1000."""
    sc = scenes.dam_break(n=1500, seed=3)
    p = sc.params
    pos = sc.pos.copy()
    escaped = np.array([5, 77, 400, 1499])
    pos[escaped[0]] = (-5000.0, 10.0, 0.0)
    pos[escaped[1]] = (0.0, -60.0, 0.0)
    pos[escaped[2]] = (np.nan, 10.0, 0.0)
    pos[escaped[3]] = (0.0, 10.0, 1e30)
    st = O.State.new(p, pos, sc.vel, sc.veval, sc.clr)
    O.insert(p, st)
    assert (st.gcell[escaped] == UNDEF).all()
    assert st.gndx[escaped].tolist() == [0, 1, 2, 3]
    assert st.cnt[-1] == 4
    O.prefix_sum(p, st)
    O.counting_sort(p, st)
    n_in = st.n - 4
    assert (st.gcell[n_in:] == UNDEF).all() and (st.gcell[:n_in] != UNDEF).all()
    assert_bit_equal(st.pos[n_in:], pos[escaped], "tail keeps index order")
    O.density(p, st)
    O.force(p, st)
    assert (st.press[n_in:] == 0).all() and (st.force[n_in:] == 0).all()
    O.advance(p, st, 0.0, p.dt, p.sim_scale)
    assert (st.pos[n_in:] == -1000.0).all() and (st.vel[n_in:] == 0).all()


def test_fp32_oracle_within_stated_tolerance_of_fp64():
    """Tier (b): FP32 density within 1e-5 relative and FP32 force within 1e-4
    of its force scale, against the FP64 restatement, one step from a
    developed (20-step) state."""
    sc = scenes.dam_break(n=8000, seed=5)
    p = sc.params
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    O.run(p, st, 20, 0.0, threads=4)
    O.insert(p, st); O.prefix_sum(p, st); O.counting_sort(p, st)
    O.density(p, st)
    m = st.gcell != UNDEF
    d64 = O.density_f64(p, st.pos, st.gcell, st.off, st.cnt)
    assert density_rel_err(st.press, d64, m, p.prest_dens) <= 1e-5
    assert density_normwise_err(st.press, d64, m) <= 1e-6
    O.force(p, st)
    f64, scale = O.force_f64(p, st.pos, st.veval, st.press, st.gcell, st.off, st.cnt)
    assert force_rel_err(st.force, f64, scale, m) <= 1e-4


def test_checker_catches_a_planted_mistake(golden_dir):
    """The comparison used everywhere must fail on a one-ulp or one-index
    change planted in the oracle's output."""
    g = np.load(golden_dir / "dam_break_2000.npz")
    p = O.params_from_bytes(g["params"])
    st = O.State.new(p, g["in_pos"], g["in_vel"], g["in_veval"], g["in_clr"])
    O.insert(p, st)
    O.prefix_sum(p, st)
    O.counting_sort(p, st)
    O.density(p, st)
    bad = st.press.copy()
    bad.view(np.uint32)[17] += 1
    with pytest.raises(AssertionError):
        assert_bit_equal(bad, g["press"], "planted density")
    gndx = st.gndx.copy()
    gndx[[3, 4]] = gndx[[4, 3]]
    if not np.array_equal(gndx, g["sort_gndx"]):
        with pytest.raises(AssertionError):
            assert_bit_equal(gndx, g["sort_gndx"], "planted gndx swap")


@pytest.mark.skipif(not O.ref_available(), reason="reference tree not present at build time")
def test_sample_volume_restatement_matches_reference_source():
    """orc_sample_volume against the reference's sampleParticles kernel body
    built for the host, on a sorted 2,000-point dam break, over boxes inside
    the scan range (the reference stores out-of-range voxels at another
    index than in-range ones)."""
    sc = scenes.dam_break(n=2000)
    p = sc.params
    R = O.RefKernels(p, sc.pos, sc.vel, sc.veval, sc.clr)
    R.insert(); R.prefix_sum(1); R.counting_sort()
    lo = np.array(p.gridMin[:], np.float32) + np.float32(1.2) / np.array(p.gridDelta[:], np.float32)
    hi = np.array(p.gridMax[:], np.float32) - np.float32(2.5) / np.array(p.gridDelta[:], np.float32)
    cnt = np.append(R.buf["gridcnt"], 0).astype(np.uint32)
    off = np.append(R.buf["gridoff"], 0).astype(np.uint32)
    for res in ((9, 7, 5), (16, 16, 16)):
        want = R.sample(res, lo, hi, 0.01)
        got = O.sample_volume(p, R.buf["pos"], off, cnt, res, lo, hi, 0.01)
        assert want.max() > 0
        assert_bit_equal(got, want, f"sample {res}")


def test_sampled_evaluations_equal_the_full_ones():
    """density_at / force_at (and their FP64 forms) evaluate chosen slots of a
    large sorted state; they must give exactly the full pass's values there."""
    sc = scenes.dam_break(n=20_000, seed=4)
    p = sc.params
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    O.run(p, st, 20, 0.0, threads=4)
    O.insert(p, st)
    O.prefix_sum(p, st)
    O.counting_sort(p, st)
    full = st.copy()
    O.density(p, full, threads=4)
    O.force(p, full, threads=4)
    idx = np.random.default_rng(0).choice(st.n, 3000, replace=False)
    assert_bit_equal(O.density_at(p, st, idx, threads=4), full.press[idx], "sampled density")
    args = (full.pos, full.veval, full.press, full.gcell, full.off, full.cnt)
    assert_bit_equal(O.force_at(p, *args, idx, threads=4), full.force[idx], "sampled force")
    d64 = O.density_f64(p, full.pos, full.gcell, full.off, full.cnt, threads=4)
    assert np.array_equal(O.density_f64_at(p, full.pos, full.gcell, full.off, full.cnt, idx, threads=4), d64[idx])
    f64, s64 = O.force_f64(p, *args, threads=4)
    fa, sa = O.force_f64_at(p, *args, idx, threads=4)
    assert np.array_equal(fa, f64[idx]) and np.array_equal(sa, s64[idx])
