"""The alternative neighbour passes against the per-point passes.

With FL_PASSES_CELL_TASKS (fl_cells.cu) the fused step walks each cell's
shared search block once per 64 of its points, in lockstep, and evaluates
the hits pair-parallel; the adjoint's rebuilt steps take their pair lists
from the cell-task density. With FL_PASSES_POINT_PAIRS (fl_pairs.cu) every
density pass walks the search block once for two points of a cell with the
same lower-band bits. FL_PASSES_AUTO switches between the per-point and
cell-task passes by the largest cell. Every point's sums keep the
reference's terms and order, so all give bit-identical states: checked over many steps on the
wave tank, on crowded cells (tasks of one cell split over many warps,
unions of thousands of candidates, groups past the pair-parallel cap; runs
of hundreds of equal points split over blocks of 1024 slots), on cells of
1..64 points (one and two points per lane), on batches, through graph
replay and fl_run_from_host (whose cell-task force pass writes the new
positions into the caller's page-locked array), through the phase entry
points, against the oracle step by step, and through the adjoint.
"""
from __future__ import annotations

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import scenes
from oracle import oracle as O

from helpers import FIELDS, assert_bit_equal

pytestmark = pytest.mark.gpu
UNDEF = 0xFFFFFFFF


ALTS = pytest.mark.parametrize("alt", ["cells", "pairs", "auto"])


def run_both(params, pos, vel, veval, clr, steps, graph=True, alt="cells"):
    out = {}
    for mode in ("points", alt):
        with F.FluidSystem(params, pos.shape[0]) as s:
            s.SetParticles(pos, vel, veval, clr=clr)
            s.SetNeighbourPasses(mode)
            assert s.NeighbourPasses() == mode
            if graph:
                s.RunSteps(steps)
            else:
                for _ in range(steps):
                    s.Run()
            s.Sync()
            assert s.IntegrityCheck() == 0
            out[mode] = s.state()
    return out["points"], out[alt]


def assert_states_equal(a, b, what):
    for k in FIELDS + ("gridcnt", "gridoff"):
        assert_bit_equal(b[k], a[k], f"{what}: {k}")


@ALTS
def test_alt_equals_points_on_the_wave_tank(alt):
    sc = scenes.wave_tank(n=300_000)
    a, b = run_both(sc.params, sc.pos, sc.vel, sc.veval, sc.clr, 40, alt=alt)
    assert_states_equal(a, b, "wave tank, 40 steps")


@ALTS
@pytest.mark.parametrize("graph", [False, True])
def test_alt_equals_points_on_the_dam_break(graph, alt):
    sc = scenes.dam_break()
    a, b = run_both(sc.params, sc.pos, sc.vel, sc.veval, sc.clr, 30, graph=graph, alt=alt)
    assert_states_equal(a, b, "dam break, 30 steps")


@ALTS
@pytest.mark.parametrize("m", [1, 31, 32, 33, 63, 64, 65, 129, 700, 3000])
def test_alt_equals_points_with_a_crowded_cell(m, alt):
    """m points packed into one cell among a dam break: tasks of 1..64
    points, a cell split into several tasks, unions of thousands; runs of
    equal points longer than a block."""
    sc = scenes.dam_break(n=6000, seed=31)
    p = sc.params
    rng = np.random.default_rng(100 + m)
    pos = sc.pos.copy()
    pick = rng.choice(pos.shape[0], size=m, replace=False)
    c = np.array([p.gridMin[0] + 7.5 * 5.0, p.gridMin[1] + 5.5 * 5.0, p.gridMin[2] + 6.5 * 5.0], np.float32)
    pos[pick] = c + rng.uniform(-2.4, 2.4, size=(m, 3)).astype(np.float32)
    a, b = run_both(p, pos, sc.vel, sc.veval, sc.clr, 4, alt=alt)
    assert_states_equal(a, b, f"crowded cell of {m}")


@ALTS
def test_alt_matches_the_oracle_step_by_step(alt):
    sc = scenes.dam_break(n=20_000, seed=4)
    p = sc.params
    with F.FluidSystem(p, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        assert s.NeighbourPasses() == "auto"   # the default
        s.SetNeighbourPasses(alt)
        s.RunSteps(40)
        s.Sync()
        for _ in range(3):
            st0 = s.state()
            ref = O.State.new(p, st0["pos"], st0["vel"], st0["veval"], st0["clr"])
            O.step(p, ref, s.time, threads=8)
            s.Run()
            s.Sync()
            st = s.state()
            for k in FIELDS:
                assert_bit_equal(st[k], getattr(ref, k), k)


@ALTS
def test_alt_equals_points_on_a_batch(alt):
    scs = scenes.batch_scenes(nscenes=12, seed=23, nmin=500, nmax=20000)
    cat = scenes.concat(scs)
    out = {}
    for mode in ("points", alt):
        with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
            b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
            b.SetNeighbourPasses(mode)
            b.RunSteps(25)
            b.Sync()
            out[mode] = b.state()
    assert_states_equal(out["points"], out[alt], "batch of 12, 25 steps")


@ALTS
def test_alt_with_escaped_points_and_nan(alt):
    sc = scenes.dam_break(n=3000, seed=12)
    pos = sc.pos.copy()
    pos[:4] = [(-500.0, 1.0, 1.0), (1.0, -300.0, 1.0), (np.nan, 0.0, 0.0), (1e30, 1e30, 1e30)]
    a, b = run_both(sc.params, pos, sc.vel, sc.veval, sc.clr, 3, alt=alt)
    assert_states_equal(a, b, "escapes")
    assert (b["gcell"] == UNDEF).sum() >= 4


def test_run_from_host_with_cells_writes_positions_back():
    """fl_run_from_host with the cell-task passes: the force pass writes the
    new positions into the caller's page-locked array as it goes; they
    equal the device state and the per-point path's step."""
    import ctypes as C
    sc = scenes.wave_tank(n=150_000)
    n = sc.n
    pins = {k: F.PinnedArray((n, 3), np.float32) for k in ("pos", "vel", "veval", "out")}
    clr = F.PinnedArray((n,), np.uint32)
    pins["pos"].array[:] = sc.pos
    pins["vel"].array[:] = sc.vel
    pins["veval"].array[:] = sc.veval
    clr.array[:] = sc.clr
    lib = F.lib()
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    try:
        with F.FluidSystem(sc.params, n) as s:
            s.SetNeighbourPasses("cells")
            pins["out"].array[:] = np.nan
            F._lib.check("fl_run_from_host", lib.fl_run_from_host(
                s.handle, n, vp(pins["pos"].array), vp(pins["vel"].array), vp(pins["veval"].array),
                vp(clr.array), vp(pins["out"].array)))
            got_host = pins["out"].array.copy()
            got = s.state()
        assert_bit_equal(got_host, got["pos"], "host copy of the new positions")
        with F.FluidSystem(sc.params, n) as s:
            s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
            s.SetNeighbourPasses("points")
            s.Run()
            s.Sync()
            want = s.state()
        for k in FIELDS:
            assert_bit_equal(got[k], want[k], f"run_from_host vs per-point step: {k}")
    finally:
        for a in list(pins.values()) + [clr]:
            a.free()


@ALTS
@pytest.mark.parametrize("every", [1, 3])
def test_adjoint_identical_with_any_passes(every, alt):
    """The adjoint's rebuilt steps take their pair lists from the selected
    density pass and its segment replays run the selected step: gradients
    must equal those of the per-point pass bit for bit."""
    sc = scenes.dam_break(n=6000, seed=41)
    w = np.random.default_rng(42).standard_normal((3, sc.n, 3)).astype(np.float32)
    got = {}
    for mode in ("points", alt):
        with F.FluidSystem(sc.params, sc.n) as s:
            s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
            s.SetNeighbourPasses(mode)
            s.RunSteps(15)
            s.TapeBegin(7, every)
            for _ in range(7):
                s.Run()
            got[mode] = s.Backward(*w)
    for k, name in enumerate(("pos", "vel", "veval")):
        assert_bit_equal(got[alt][k], got["points"][k], f"every={every}: dL/d{name}")
    assert np.array_equal(got[alt][3], got["points"][3])


@pytest.mark.parametrize("n", [1, 2, 1023, 1024, 1025, 5000])
def test_pairs_through_the_phase_entry_points(n):
    """The reference's phase sequence (insert, prefix sum, counting sort,
    ComputePressure, ComputeForce, Advance) with the paired density: the
    same densities, pair lists and forces as the per-point pass, at sizes
    around the pass's 1024-slot blocks."""
    sc = scenes.dam_break(n=max(n, 2), seed=7)
    pos, vel, veval, clr = sc.pos[:n], sc.vel[:n], sc.veval[:n], sc.clr[:n]
    if n == 2:   # two points of one cell with the same band bits: one item
        pos = np.array([[0.0, 0.0, 0.0]], np.float32) + sc.pos[:1]
        pos = np.concatenate([pos, pos + np.float32(0.01)])
    out = {}
    for mode in ("points", "pairs"):
        with F.FluidSystem(sc.params, n) as s:
            s.SetParticles(pos, vel, veval, clr=clr)
            s.SetNeighbourPasses(mode)
            for _ in range(3):
                s.InsertParticlesCUDA()
                s.PrefixSumCellsCUDA(1)
                s.CountingSortFullCUDA()
                s.ComputePressureCUDA()
                s.ComputeForceCUDA()
                s.AdvanceCUDA(s.time, sc.params.dt, sc.params.sim_scale)
            s.Sync()
            out[mode] = s.state()
    assert_states_equal(out["points"], out["pairs"], f"phase sequence, n={n}")


def test_auto_switches_to_cell_tasks_when_a_cell_crowds_and_back():
    """FL_PASSES_AUTO: the per-point passes while every cell is small, the
    cell tasks once the largest in-range cell passes 512 points (acting on
    the count a step or two late), the per-point passes again below 384;
    points out of range (the bin) do not count. The states equal the
    per-point passes' at every stage."""
    sc = scenes.dam_break(n=8000, seed=71)
    p = sc.params
    rng = np.random.default_rng(72)
    crowded = sc.pos.copy()
    c = np.array([p.gridMin[0] + 7.5 * 5.0, p.gridMin[1] + 5.5 * 5.0, p.gridMin[2] + 6.5 * 5.0], np.float32)
    crowded[:1500] = c + rng.uniform(-2.4, 2.4, size=(1500, 3)).astype(np.float32)
    escaped = sc.pos.copy()
    escaped[:2000] = (-500.0, 1.0, 1.0)
    for name, pos, want in (("small cells", sc.pos, "points"), ("escaped", escaped, "points"),
                            ("crowded", crowded, "cells")):
        out = {}
        for mode in ("points", "auto"):
            with F.FluidSystem(p, sc.n) as s:
                s.SetParticles(pos, sc.vel, sc.veval, clr=sc.clr)
                s.SetNeighbourPasses(mode)
                s.RunSteps(3)
                s.Sync()
                for _ in range(2):   # the recorded count reaches the host
                    s.Run()
                s.Sync()
                if mode == "auto":
                    assert s.NeighbourPassesInUse() == want, name
                s.RunSteps(6)   # graph replays in the selected passes
                s.Sync()
                out[mode] = s.state()
        assert_states_equal(out["points"], out["auto"], name)
    # back to the per-point passes once the crowd is gone
    with F.FluidSystem(p, sc.n) as s:
        s.SetParticles(crowded, sc.vel, sc.veval, clr=sc.clr)
        s.RunSteps(3)
        s.Run(); s.Run(); s.Sync()
        assert s.NeighbourPassesInUse() == "cells"
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        for _ in range(4):
            s.Run()
        s.Sync()
        assert s.NeighbourPassesInUse() == "points"


def test_auto_switches_within_one_long_call():
    """One RunSteps call of 100 steps with FL_PASSES_AUTO runs in chunks of
    32 steps, each chunk's passes chosen from the counts of the chunk two
    before it: a crowd that forms switches the call to the cell tasks
    midway, with the per-point passes' states."""
    sc = scenes.dam_break(n=8000, seed=73)
    p = sc.params
    rng = np.random.default_rng(74)
    pos = sc.pos.copy()
    c = np.array([p.gridMin[0] + 7.5 * 5.0, p.gridMin[1] + 5.5 * 5.0, p.gridMin[2] + 6.5 * 5.0], np.float32)
    pos[:3000] = c + rng.uniform(-2.4, 2.4, size=(3000, 3)).astype(np.float32)
    out = {}
    for mode in ("points", "auto"):
        with F.FluidSystem(p, sc.n) as s:
            s.SetParticles(pos, sc.vel, sc.veval, clr=sc.clr)
            s.SetNeighbourPasses(mode)
            before = s.PassesSteps()
            s.RunSteps(100)
            s.Sync()
            points_steps, cell_steps = (a - b for a, b in zip(s.PassesSteps(), before))
            assert points_steps + cell_steps == 100
            if mode == "auto":   # the call began with the per-point passes and switched
                assert points_steps >= 32 and cell_steps >= 32, (points_steps, cell_steps)
            assert s.IntegrityCheck() == 0
            out[mode] = s.state()
    assert_states_equal(out["points"], out["auto"], "100 steps in one call")


def test_passes_and_reverse_list_modes_reject_unknown_values():
    sc = scenes.dam_break(n=500)
    lib = F.lib()
    with F.FluidSystem(sc.params, sc.n) as s:
        for bad in (-1, 4, 99):
            assert lib.fl_set_neighbour_passes(s.handle, bad) == -1          # FL_ERR_ARG
            assert lib.fl_set_reverse_lists(s.handle, bad if bad != 4 else 3) == -1
        assert s.NeighbourPasses() == "auto"
        assert s.PassesSteps() == (0, 0)
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        s.RunSteps(3)
        s.Sync()
        assert s.PassesSteps() == (3, 0)
        s.SetNeighbourPasses("cells")
        s.RunSteps(2)
        s.Sync()
        assert s.PassesSteps() == (3, 2)
        assert s.NeighbourPassesInUse() == "cells"
