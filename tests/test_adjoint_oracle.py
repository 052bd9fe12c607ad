"""CPU tests of the FP64 adjoint model (oracle/adjoint64.c).

The model is the SPH step with its integer structure -- the per-step sort
permutation, the in-range flags and the neighbour pairs -- frozen from an
FP32 oracle run, evaluated in double. Its hand-written reverse pass is
checked here against central finite differences of its own forward, for
directional derivatives along random directions of the initial positions,
velocities, evaluated velocities and of (viscosity, rest density,
IntStiff). The GPU adjoint is then checked against this model.
"""
from __future__ import annotations

import numpy as np
import pytest

from fluids3_gb300 import scenes
from oracle import oracle as O

from helpers import stirred_state as _stirred_state


def _fd_check(p, fz, seed, rel_tol=1e-5):
    rng = np.random.default_rng(seed)
    n = fz.n
    x0, v0, e0 = (np.array(a) for a in fz.states[0])
    wx, wv, we = rng.standard_normal((3, n, 3))
    th0 = np.array([p.pvisc, p.prest_dens, p.pintstiff], np.float64)

    def loss(x, v, e, th=th0):
        xf, vf, ef = O.adj64_forward(p, fz, x, v, e, th)
        return (wx * xf).sum() + (wv * vf).sum() + (we * ef).sum()

    gx, gv, ge, gp = O.adj64_backward(p, fz, wx, wv, we, x0, v0, e0, theta=th0, use_states=False)
    base = [x0, v0, e0]
    for k, g in enumerate((gx, gv, ge)):
        d = rng.standard_normal((n, 3))
        eps = 1e-6
        ap = list(base); ap[k] = base[k] + eps * d
        am = list(base); am[k] = base[k] - eps * d
        fd = (loss(*ap) - loss(*am)) / (2 * eps)
        an = float((g * d).sum())
        assert abs(fd - an) <= rel_tol * max(abs(fd), 1e-3), ("xve"[k], fd, an)
    for k in range(3):
        eps = 1e-6 * max(1.0, abs(th0[k]))
        tp = th0.copy(); tp[k] += eps
        tm = th0.copy(); tm[k] -= eps
        fd = (loss(x0, v0, e0, tp) - loss(x0, v0, e0, tm)) / (2 * eps)
        assert abs(fd - gp[k]) <= rel_tol * max(abs(fd), 1e-3), ("theta", k, fd, gp[k])


def test_adjoint64_matches_finite_differences_dam_break():
    sc = scenes.dam_break(n=2000)
    st, t = _stirred_state(sc, 20, seed=1)
    fz = O.frozen_run(sc.params, st, 3, t)
    assert fz.pnbr.size > 10 * fz.n       # a real neighbourhood
    _fd_check(sc.params, fz, seed=2)


def test_adjoint64_matches_finite_differences_moving_wall_and_slope():
    sc = scenes.wave_tank(n=3000)
    p = sc.params
    p.bound_slope = 0.05   # sloped floor (fluid_kernels.cu:356) on top of the moving X- wall
    st, t = _stirred_state(sc, 0, seed=3)
    fz = O.frozen_run(p, st, 4, 1.7)
    _fd_check(p, fz, seed=4)


def test_adjoint64_out_of_range_points_pass_only_veval():
    # A point outside the scan range is parked at -1000 with zero velocity;
    # its evaluated velocity carries over, so only that adjoint survives.
    sc = scenes.dam_break(n=500)
    p = sc.params
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    st.pos[7] = (1.0e4, 1.0e4, 1.0e4)
    st.veval[7] = (0.5, -0.25, 0.125)
    fz = O.frozen_run(p, st, 1, 0.0)
    slot = int(np.nonzero(fz.perm[0] == 7)[0][0])
    assert fz.inr[0, slot] == 0
    n = fz.n
    xb, vb, eb = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    xb[slot], vb[slot], eb[slot] = (1.0, 2.0, 3.0), (4.0, 5.0, 6.0), (7.0, 8.0, 9.0)
    gx, gv, ge, gp = O.adj64_backward(p, fz, xb, vb, eb)
    assert np.all(gx[7] == 0) and np.all(gv[7] == 0)
    assert ge[7].tolist() == [7.0, 8.0, 9.0]
    assert np.count_nonzero(gx) == 0 and np.count_nonzero(gv) == 0
    assert np.all(gp == 0)


@pytest.mark.parametrize("steps", [1, 5])
def test_adjoint64_linearised_at_fp32_states_is_close_to_its_own(steps):
    # Linearising around the recorded FP32 trajectory (what the GPU adjoint
    # does) differs from linearising around the FP64 forward only by the
    # FP32-vs-FP64 state difference.
    sc = scenes.dam_break(n=1500)
    st, t = _stirred_state(sc, 10, seed=5)
    fz = O.frozen_run(sc.params, st, steps, t)
    rng = np.random.default_rng(6)
    w = rng.standard_normal((3, fz.n, 3))
    a = O.adj64_backward(sc.params, fz, *w, use_states=True)
    x0, v0, e0 = fz.states[0]
    b = O.adj64_backward(sc.params, fz, *w, x0, v0, e0, use_states=False)
    for ga, gb in zip(a, b):
        assert np.linalg.norm(ga - gb) <= 1e-3 * np.linalg.norm(gb) + 1e-12


def _final_order(fz):
    order = np.arange(fz.n, dtype=np.int64)
    for k in range(fz.steps):
        order = order[fz.perm[k]]
    return order


def rollout_loss64(p, fz, target, x0, v0, e0, theta, masks=None, mask_mode=0):
    """The differentiated rollout's loss (mean squared distance of the final
    positions to the target, over the points in range at the last step) on
    the FP64 frozen-structure model, and its cotangent on the final state."""
    x, _, _ = O.adj64_forward(p, fz, x0, v0, e0, theta, masks, mask_mode)
    live = fz.inr[-1].astype(bool)
    d = np.where(live[:, None], x - target[_final_order(fz)], 0.0)
    m = int(live.sum())
    return float((d ** 2).sum()) / m, 2.0 * d / m


def test_rollout_65k_gradient_matches_central_differences():
    """The 65,536-point scaled dam break, 8 steps: the loss gradient with
    respect to (viscosity, rest density, IntStiff) and along a random
    direction of the initial velocity field, adjoint against central
    differences, both on the FP64 model. Parameters: a step of 1e-4
    relative with the wall and limit decisions frozen as well (over 65,536
    points some point sits within 1e-4 of a threshold, where the model has a
    kink), and 1e-6 relative with free decisions. Velocity field: the loss
    curves strongly along a 196,608-dimensional direction (central
    differences converge quadratically: 2.5e-2 off at a step of 1e-4, 2.5e-4
    at 1e-5), so the steps there are 1e-5 (frozen) and 1e-7 (free)."""
    sc = scenes.dam_break_scaled(65536)
    p = sc.params
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    t = O.run(p, st, 20, 0.0, threads=4)           # a moving state, not the lattice at rest
    fz = O.frozen_run(p, st.copy(), 8, t)
    target = scenes.shifted_target(sc)
    x0, v0, e0 = (np.array(a) for a in fz.states[0])
    th0 = np.array([p.pvisc, p.prest_dens, p.pintstiff], np.float64)
    masks = np.zeros((fz.steps, fz.n), np.uint8)
    loss, cot = rollout_loss64(p, fz, target, x0, v0, e0, th0, masks, 1)
    gx, gv, ge, gp = O.adj64_backward(p, fz, cot, np.zeros_like(cot), np.zeros_like(cot), x0, v0, e0,
                                      theta=th0, use_states=False)
    d = np.random.default_rng(8).standard_normal(v0.shape)
    for rel, hv, mode in ((1e-4, 1e-5, 2), (1e-6, 1e-7, 0)):
        L = lambda th, v: rollout_loss64(p, fz, target, x0, v, e0, th, masks, mode)[0]
        for k in range(3):
            h = rel * abs(th0[k])
            tp = th0.copy(); tp[k] += h
            tm = th0.copy(); tm[k] -= h
            fd = (L(tp, v0) - L(tm, v0)) / (2 * h)
            assert abs(fd - gp[k]) <= 1e-3 * abs(fd), ("param", k, rel, fd, gp[k])
        fd = (L(th0, v0 + hv * d) - L(th0, v0 - hv * d)) / (2 * hv)
        an = float((gv * d).sum())
        assert abs(fd - an) <= 1e-3 * abs(fd), ("velocity", hv, fd, an)
