"""Shared checks for the parity tests."""
from __future__ import annotations

import hashlib

import numpy as np

FIELDS = ("pos", "vel", "veval", "force", "press", "clr", "gcell", "gndx")


def bits(a: np.ndarray) -> np.ndarray:
    """The raw 32-bit patterns (bit-exact comparison, NaN-safe)."""
    a = np.ascontiguousarray(a)
    return a.view(np.uint32)


def assert_bit_equal(got: np.ndarray, want: np.ndarray, what: str) -> None:
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, f"{what}: shape {got.shape} != {want.shape}"
    g, w = bits(got).reshape(-1), bits(want).reshape(-1)
    bad = np.nonzero(g != w)[0]
    if bad.size:
        k = bad[0]
        raise AssertionError(f"{what}: {bad.size} of {g.size} words differ; first at flat index {k}: "
                             f"{got.reshape(-1)[k]!r} != {want.reshape(-1)[k]!r}")


def digest(buf: dict) -> str:
    h = hashlib.sha256()
    for k in FIELDS:
        h.update(np.ascontiguousarray(buf[k]).tobytes())
    return h.hexdigest()


def density_rel_err(got, ref64, mask, rest_density: float) -> float:
    """Max relative error of densities against the FP64 oracle over the points
    whose density is at least a tenth of the rest density.

    Below that a point is an isolated splash whose few pair terms all sit at
    the support cutoff, where (rd2 - d^2) cancels: the reference's FP32
    formula itself loses digits there (any FP32 evaluation does), so those
    points are held to bit-equality with the FP32 reference path instead.
    The norm-wise error over all points is checked separately."""
    g = np.asarray(got, np.float64)
    r = np.asarray(ref64, np.float64)
    m = mask & (r >= 0.1 * rest_density)
    return float(np.max(np.abs(g[m] - r[m]) / np.abs(r[m]))) if m.any() else 0.0


def density_normwise_err(got, ref64, mask) -> float:
    g = np.asarray(got, np.float64)[mask]
    r = np.asarray(ref64, np.float64)[mask]
    return float(np.linalg.norm(g - r) / np.linalg.norm(r)) if r.size else 0.0


def force_rel_err(got, ref64, scale64, mask) -> float:
    """Max per-point force error against the FP64 oracle, relative to the
    point's force scale: the sum of the magnitudes of its pair terms (an
    FP32 sum's error is bounded by a multiple of that, even when the terms
    cancel)."""
    g = np.asarray(got, np.float64)[mask]
    r = np.asarray(ref64, np.float64)[mask]
    s = np.asarray(scale64, np.float64)[mask]
    err = np.linalg.norm(g - r, axis=1)
    s = np.where(s > 0, s, 1.0)
    return float(np.max(err / s)) if r.size else 0.0


def stirred_state(sc, warm_steps, seed):
    """A scene advanced `warm_steps` FP32 oracle steps, then stirred so that
    every branch of the advance is taken: some velocities above the speed
    limit, some points pushed against every wall."""
    from oracle import oracle as O
    p = sc.params
    st = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    t = O.run(p, st, warm_steps, 0.0) if warm_steps else 0.0
    rng = np.random.default_rng(seed)
    n = st.n
    fast = rng.choice(n, n // 20, replace=False)
    st.vel[fast] *= np.float32(1.0)
    st.vel[fast] += rng.normal(0.0, 3.0, (fast.size, 3)).astype(np.float32)
    lo = np.array(p.bound_min, np.float32)
    hi = np.array(p.bound_max, np.float32)
    wall = rng.choice(n, 12, replace=False)
    for k, i in enumerate(wall):
        ax = k % 3
        low = (k // 3) % 2 == 0
        st.pos[i, ax] = (lo[ax] + np.float32(0.3)) if low else (hi[ax] - np.float32(0.3))
        # moving into the wall: the damping term pushes |accel| past AccelLimit
        st.veval[i, ax] = np.float32(-2.0 if low else 2.0) if k < 6 else np.float32(0.0)
    return st, t
