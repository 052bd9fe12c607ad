"""GPU adjoint of the fused step (fl_tape_begin / fl_backward) against the
FP64 frozen-structure adjoint of the oracle (oracle/adjoint64.c), whose own
reverse pass is checked against finite differences on the CPU.

The GPU runs the recorded steps; the oracle takes each step's structure
(sort permutation, pairs) from the state the GPU had before that step and
linearises around the same states, so the two adjoints differ only by
FP32-versus-FP64 evaluation of the same formulas. Tolerance: norm-wise
relative error <= 2e-4 on each state gradient and <= 1e-3 on each
parameter gradient.
"""
from __future__ import annotations

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import _lib, scenes
from oracle import oracle as O

from helpers import assert_bit_equal, stirred_state

pytestmark = pytest.mark.gpu

STATE_TOL = 2e-4
PARAM_TOL = 1e-3
FL_ERR_ARG, FL_ERR_CAPACITY, FL_ERR_STATE = -1, -4, -6   # include/fluids_gb300.h


def _gpu_record(sc, st, time, steps, every, params=None, keep_lists=False):
    """Run `steps` taped GPU steps from oracle state `st`; returns the system
    (still open) and the per-step (pos, vel, veval) read back before each step."""
    p = params or sc.params
    s = F.FluidSystem(p, st.n)
    s.SetParticles(st.pos, st.vel, st.veval, clr=st.clr)
    s.time = time
    s.TapeBegin(steps, every, keep_lists)
    states = []
    for _ in range(steps):
        states.append((s.GetBuffer(F.FPOS), s.GetBuffer(F.FVEL), s.GetBuffer(F.FVEVAL)))
        s.Run()
    s.Sync()
    return s, states


def _oracle_adjoint(p, st, states, time, steps, w):
    times = [float(np.float32(time))]
    for _ in range(steps - 1):
        times.append(float(np.float32(np.float32(times[-1]) + np.float32(p.dt))))
    fz = O.frozen_run(p, st.copy(), steps, time, states=states, times=times)
    return O.adj64_backward(p, fz, *w, use_states=True), fz


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


def _check(got, want):
    gx, gv, ge, gp = got
    wx, wv, we, wp = want
    errs = {"pos": _rel(gx, wx), "vel": _rel(gv, wv), "veval": _rel(ge, we)}
    for k, e in errs.items():
        assert e <= STATE_TOL, (k, errs)
    for k in range(3):
        e = abs(gp[0, k] - wp[k]) / max(abs(wp[k]), 1e-30)
        assert e <= PARAM_TOL, ("param", k, gp[0, k], wp[k])
    return errs


@pytest.mark.parametrize("steps,every", [(1, 1), (4, 1), (5, 2)])
def test_backward_matches_fp64_adjoint_dam_break(steps, every):
    sc = scenes.dam_break(n=2000)
    st, t = stirred_state(sc, 20, seed=11)
    s, states = _gpu_record(sc, st, t, steps, every)
    rng = np.random.default_rng(12)
    w = rng.standard_normal((3, st.n, 3)).astype(np.float32)
    with s:
        assert s.TapeSteps() == steps
        got = s.Backward(*w)
    want, _ = _oracle_adjoint(sc.params, st, states, t, steps, w)
    _check(got, want)


def test_backward_matches_fp64_adjoint_moving_wall_slope_and_crowding():
    sc = scenes.wave_tank(n=6000)
    p = sc.params
    p.bound_slope = 0.05
    st, t = stirred_state(sc, 0, seed=13)
    # a crowd of 1,200 points within one smoothing radius: their pair lists
    # (128 entries) overflow and both passes walk for them
    rng = np.random.default_rng(14)
    st.pos[:1200] = st.pos[1300] + rng.uniform(-0.6, 0.6, (1200, 3)).astype(np.float32)
    s, states = _gpu_record(sc, st, 1.7, 3, 1, params=p)
    w = rng.standard_normal((3, st.n, 3)).astype(np.float32)
    with s:
        got = s.Backward(*w)
    want, _ = _oracle_adjoint(p, st, states, 1.7, 3, w)
    _check(got, want)


@pytest.mark.parametrize("grid_density,srch", [(2.0, 3), (3.0, 5)])
def test_backward_wider_search_blocks(grid_density, srch):
    # no pruning; reverse blocks c-(srch-2) .. c+1, clipped to the scan range
    sc = scenes.dam_break(n=1500)
    p = scenes.make_params((-30.0, 0.0, -30.0), (30.0, 60.0, 30.0), grid_density=grid_density)
    assert p.gridSrch == srch
    st, t = stirred_state(scenes.Scene("g3", p, sc.pos, sc.vel, sc.veval, sc.clr), 5, seed=15)
    s, states = _gpu_record(sc, st, t, 3, 1, params=p)
    w = np.random.default_rng(16).standard_normal((3, st.n, 3)).astype(np.float32)
    with s:
        got = s.Backward(*w)
    want, _ = _oracle_adjoint(p, st, states, t, 3, w)
    _check(got, want)


def test_backward_escaped_points_and_tape_order():
    sc = scenes.dam_break(n=1200)
    st, t = stirred_state(sc, 3, seed=17)
    p = sc.params
    st.pos[5] = (1.0e4, 1.0e4, 1.0e4)          # out of range from the start
    # just inside the first scanned x cell, moving out at the speed limit
    # (3 * dt / ss = 2.25 units per step): it leaves the scan range
    st.pos[9] = (p.gridMin[0] + np.float32(1.0) / p.gridDelta[0] + np.float32(0.5), 30.0, 0.0)
    st.vel[9] = (-3.0, 0.0, 0.0)
    st.veval[9] = (-3.0, 0.0, 0.0)
    s, states = _gpu_record(sc, st, t, 4, 1)
    w = np.random.default_rng(18).standard_normal((3, st.n, 3)).astype(np.float32)
    with s:
        order = s.TapeOrder()
        got = s.Backward(*w)
    want, fz = _oracle_adjoint(sc.params, st, states, t, 4, w)
    ident = np.arange(st.n, dtype=np.uint32)
    for k in range(4):
        ident = ident[fz.perm[k]]
    assert_bit_equal(order, ident, "tape order")
    assert fz.inr[0].sum() == st.n - 1 and fz.inr[-1].sum() < st.n - 1   # one escaped on the way
    _check(got, want)
    assert got[0][5].tolist() == [0.0, 0.0, 0.0] and got[1][5].tolist() == [0.0, 0.0, 0.0]


def test_checkpoint_segments_and_repeat_are_bit_identical():
    sc = scenes.dam_break(n=4000)
    st, t = stirred_state(sc, 15, seed=19)
    w = np.random.default_rng(20).standard_normal((3, st.n, 3)).astype(np.float32)
    results = []
    for every, keep in ((1, False), (3, False), (7, False), (1, True), (3, True), (7, True)):
        s, _ = _gpu_record(sc, st, t, 7, every, keep_lists=keep)
        with s:
            a = s.Backward(*w)
            b = s.Backward(*w)
            for x, y in zip(a, b):
                assert_bit_equal(x, y, f"repeat, every={every}, keep_lists={keep}")
            results.append(a)
    for r in results[1:]:
        for x, y in zip(results[0], r):
            assert_bit_equal(x, y, "every=1 vs segmented")


def test_backward_leaves_the_run_untouched():
    sc = scenes.dam_break(n=3000)
    st, t = stirred_state(sc, 5, seed=21)
    a = F.FluidSystem(sc.params, st.n)
    b = F.FluidSystem(sc.params, st.n)
    with a, b:
        for s in (a, b):
            s.SetParticles(st.pos, st.vel, st.veval, clr=st.clr)
            s.time = t
        a.TapeBegin(10, 2)
        a.RunSteps(5)
        b.RunSteps(5)
        before = a.state()
        a.Backward(np.ones((st.n, 3), np.float32))
        after = a.state()
        for k in ("pos", "vel", "veval", "force", "press", "clr", "gcell", "gndx"):
            assert_bit_equal(after[k], before[k], k)
        assert a.time == b.time
        a.RunSteps(3)     # still recording: steps 6..8 join the tape
        b.RunSteps(3)
        assert a.TapeSteps() == 8
        for k in (F.FPOS, F.FVEL, F.FVEVAL):
            assert_bit_equal(a.GetBuffer(k), b.GetBuffer(k), f"buffer {k}")


def test_backward_is_linear_in_the_cotangent():
    sc = scenes.wave_tank(n=200_000)
    s = F.FluidSystem(sc.params, sc.n)
    with s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        s.RunSteps(20)
        s.TapeBegin(6, 3)
        s.RunSteps(6)
        rng = np.random.default_rng(22)
        w1 = rng.standard_normal((3, sc.n, 3)).astype(np.float32)
        w2 = rng.standard_normal((3, sc.n, 3)).astype(np.float32)
        g1 = s.Backward(*w1)
        g2 = s.Backward(*w2)
        g12 = s.Backward(*(2.0 * w1 + w2))
    for k in range(3):
        want = 2.0 * g1[k].astype(np.float64) + g2[k]
        assert _rel(g12[k], want) <= 1e-5, k
    want = 2.0 * g1[3] + g2[3]
    assert np.all(np.abs(g12[3] - want) <= 1e-4 * np.abs(want) + 1e-9)


@pytest.mark.parametrize("crowd", [False, True])
def test_batched_backward_equals_each_scene_alone(crowd):
    """Gradients of each scene in a batch equal the scene's alone, bit for
    bit; with crowd, 300 points of each scene cluster so their pair lists
    overflow and the crowd kernel walks them (scene slot bases are not
    multiples of 32 here)."""
    scs = scenes.batch_scenes(nscenes=3, nmin=1500, nmax=4000, seed=23)
    for k, sc in enumerate(scs):
        sc.vel[:] = np.float32(0.1 * (k + 1))
        if crowd:
            c = sc.pos[sc.n // 2].copy()
            sc.pos[:300] = c + np.random.default_rng(40 + k).uniform(-0.5, 0.5, (300, 3)).astype(np.float32)
    rng = np.random.default_rng(24)
    ws = [rng.standard_normal((3, sc.n, 3)).astype(np.float32) for sc in scs]
    alone = []
    for sc, w in zip(scs, ws):
        with F.FluidSystem(sc.params, sc.n) as s:
            s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
            s.RunSteps(4)
            s.TapeBegin(4, 2)
            s.RunSteps(4)
            alone.append(s.Backward(*w))
    cat = scenes.concat(scs)
    with F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        b.RunSteps(4)
        b.TapeBegin(4, 2)
        b.RunSteps(4)
        got = b.Backward(*[np.concatenate([w[j] for w in ws]) for j in range(3)])
    base = 0
    for k, (sc, a) in enumerate(zip(scs, alone)):
        for j in range(3):
            assert_bit_equal(got[j][base:base + sc.n], a[j], f"scene {k} grad {j}")
        assert_bit_equal(got[3][k], a[3][0], f"scene {k} params")
        base += sc.n


def test_tape_errors():
    sc = scenes.dam_break(n=500)
    with F.FluidSystem(sc.params, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        lib = _lib.lib()
        assert lib.fl_backward(s.handle, None, None, None, None, None, None, None) == FL_ERR_STATE
        s.TapeBegin(2)
        assert lib.fl_backward(s.handle, None, None, None, None, None, None, None) == FL_ERR_STATE
        s.Run(); s.Run()
        assert lib.fl_run(s.handle) == FL_ERR_CAPACITY      # tape full
        s.SetParticles(sc.pos, sc.vel, sc.veval)               # state replaced mid-tape
        assert lib.fl_backward(s.handle, None, None, None, None, None, None, None) == FL_ERR_STATE
        assert b"changed outside Run" in lib.fl_last_error()
        assert lib.fl_tape_begin(s.handle, 0, 1) == FL_ERR_ARG
        assert lib.fl_tape_begin(s.handle, 4, 5) == FL_ERR_ARG
        s.TapeBegin(3, 3)
        s.RunSteps(3)
        gx, gv, ge, gp = s.Backward()                            # zero cotangent
        assert not gx.any() and not gv.any() and not ge.any() and not gp.any()
        s.TapeEnd()
        assert s.TapeSteps() == 0


def test_differentiated_rollout_65k_against_fp64_adjoint():
    """The differentiated rollout on the 65,536-point scaled dam break (8
    steps, checkpoints every 4): loss on the final positions against the
    shifted target cloud; gradients with respect to the initial state and
    (viscosity, rest density, IntStiff) against the FP64 adjoint on the same
    trajectory (the forward here is bit-identical to the oracle's)."""
    from fluids3_gb300.rollout import differentiated_rollout
    sc = scenes.dam_break_scaled(65536)
    p = sc.params
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    t = O.run(p, st, 20, 0.0, threads=4)
    target = scenes.shifted_target(sc)
    with F.FluidSystem(p, st.n) as s:
        s.SetParticles(st.pos, st.vel, st.veval, clr=st.clr)
        s.time = t
        r = differentiated_rollout(s, 8, target, every=4)
    fz = O.frozen_run(p, st.copy(), 8, t)
    order = np.arange(st.n)
    for k in range(8):
        order = order[fz.perm[k]]
    assert_bit_equal(r["order"], order.astype(np.uint32), "final order")
    cot = r["dloss_dpos"]
    want = O.adj64_backward(p, fz, cot, np.zeros_like(cot), np.zeros_like(cot), use_states=True)
    _check((r["grad_pos"], r["grad_vel"], r["grad_veval"], r["grad_params"]), want)
    assert r["points"] == int(fz.inr[-1].sum()) and r["loss"] > 0


def test_long_rollout_gradient_stays_finite_and_matches_fp64():
    """300 steps of the 2,000-point dam break: the exact gradient grows
    ~1.4x per step to ~1e44, beyond FP32. fl_backward_scaled renormalises
    the cotangents by powers of two during the reverse pass and returns
    mantissas with a binary exponent; mantissa * 2^exponent must match the
    FP64 adjoint (linearised around the same recorded states), while the
    plain fl_backward overflows float."""
    sc = scenes.dam_break(n=2000, seed=4)
    st = O.State.new(sc.params, sc.pos, sc.vel, sc.veval, sc.clr)
    steps = 300
    s, states = _gpu_record(sc, st, 0.0, steps, 20)
    w = np.random.default_rng(19).standard_normal((3, st.n, 3)).astype(np.float32)
    with s:
        gx, gv, ge, gp, ex = s.BackwardScaled(*w)
        plain = s.Backward(*w)
    assert ex.shape == (1,) and ex[0] > 60
    scale = 2.0 ** int(ex[0])
    got = (gx.astype(np.float64) * scale, gv.astype(np.float64) * scale, ge.astype(np.float64) * scale, gp)
    for a in got:
        assert np.isfinite(a).all()
    assert not np.isfinite(plain[1]).all()          # the float result itself overflows
    want, _ = _oracle_adjoint(sc.params, st, states, 0.0, steps, w)
    errs = {k: _rel(got[i], want[i]) for i, k in enumerate(("pos", "vel", "veval"))}
    for k, e in errs.items():
        assert e <= 1e-3, (k, errs)
    for k in range(3):
        assert abs(gp[0, k] - want[3][k]) <= 1e-3 * abs(want[3][k]), ("param", k, gp[0, k], want[3][k])
    print(f"\n300-step gradient: exponent {int(ex[0])}, relative errors {errs}")


def _reverse_lists_both_ways(make, w, every=2):
    """Gradients with the reverse lists transposed from the pair lists and
    walked (fl_set_reverse_lists), from the same recording."""
    out = []
    for mode in (2, 1):   # FL_REVERSE_TRANSPOSE, FL_REVERSE_WALK
        with make() as s:
            s.RunSteps(5)
            _lib.check("fl_set_reverse_lists", _lib.lib().fl_set_reverse_lists(s.handle, mode))
            s.TapeBegin(4, every)
            s.RunSteps(4)
            out.append(s.Backward(*w))
    return out


@pytest.mark.parametrize("case", ["wave", "crowd", "keep_lists", "srch3", "batch"])
def test_reverse_lists_transposed_equal_walked(case):
    """The reverse pair lists are the density pass's pair lists transposed
    and sorted into ascending slot order; the walk of each point's reverse
    block finds the same lists, so every gradient is bit-identical: on the
    wave tank, with a crowd whose lists overflow (owners walk their blocks
    again, reverse counts clamp to the overflow mark), with kept lists, with
    a wider (unpruned) search block, and in a batch."""
    rng = np.random.default_rng(61)
    if case == "batch":
        scs = scenes.batch_scenes(nscenes=3, nmin=1500, nmax=4000, seed=62)
        c = scs[1].pos[scs[1].n // 2].copy()
        scs[1].pos[:400] = c + rng.uniform(-0.5, 0.5, (400, 3)).astype(np.float32)
        cat = scenes.concat(scs)

        def make():
            b = F.FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs])
            b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
            return b
        n = cat["pos"].shape[0]
    else:
        sc = scenes.wave_tank(n=8000) if case != "srch3" else scenes.dam_break(n=3000)
        p = sc.params
        if case == "srch3":
            p = scenes.make_params((-30.0, 0.0, -30.0), (30.0, 60.0, 30.0), grid_density=2.0)
            assert p.gridSrch == 3
        pos = sc.pos.copy()
        if case == "crowd":
            pos[:1500] = pos[2000] + rng.uniform(-0.6, 0.6, (1500, 3)).astype(np.float32)

        def make():
            s = F.FluidSystem(p, sc.n)
            s.SetParticles(pos, sc.vel, sc.veval, clr=sc.clr)
            return s
        n = sc.n
    w = rng.standard_normal((3, n, 3)).astype(np.float32)
    if case == "keep_lists":
        out = []
        for mode in (2, 1):   # FL_REVERSE_TRANSPOSE, FL_REVERSE_WALK
            with make() as s:
                s.RunSteps(5)
                _lib.check("fl_set_reverse_lists", _lib.lib().fl_set_reverse_lists(s.handle, mode))
                s.TapeBegin(4, 2, True)
                s.RunSteps(4)
                out.append(s.Backward(*w))
    else:
        out = _reverse_lists_both_ways(make, w)
    for j in range(3):
        assert np.isfinite(out[0][j]).all()
        assert_bit_equal(out[0][j], out[1][j], f"{case}: state gradient {j}")
    assert np.array_equal(out[0][3], out[1][3]), f"{case}: parameter gradients"
