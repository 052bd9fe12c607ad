"""Differentiated rollouts over the adjoint C ABI (fl_tape_begin / fl_backward).

A rollout runs `steps` fused steps while the tape records, forms a loss on
the final positions, and takes its gradient with respect to the initial
particle state and to (viscosity, rest density, IntStiff) -- per scene for
a batched system. No counterpart in the reference, whose step has no
derivative.
"""
from __future__ import annotations

import numpy as np

from .system import FGCELL, FPOS, GRID_UNDEF, FluidSystem

PARAM_NAMES = ("pvisc", "prest_dens", "pintstiff")


def position_loss(system: FluidSystem, target: np.ndarray, order: np.ndarray | None = None):
    """Mean squared distance (world units^2) of the final positions to
    `target` (per point, indexed as when recording began), over the points
    that were inside the scan range at the start of the last step (the others
    are parked at -1000 and carry no derivative) and whose target is finite
    (NaN marks a point without one). Returns (loss, dL/dpos in
    the current slot order as float32, number of points counted); for a
    batched system the mean is taken per scene and the losses summed."""
    if order is None:
        order = system.TapeOrder()
    x = system.GetBuffer(FPOS).astype(np.float64)
    y = np.asarray(target, np.float64)[order]
    live = (system.GetBuffer(FGCELL) != GRID_UNDEF) & np.isfinite(y).all(axis=1) & np.isfinite(x).all(axis=1)
    d = np.where(live[:, None], np.where(live[:, None], x, 0.0) - np.where(np.isfinite(y), y, 0.0), 0.0)
    grad = np.zeros_like(d)
    loss = 0.0
    counted = 0
    for scene in range(system.NumScenes()):
        info = system.SceneInfo(scene) if system.NumScenes() > 1 else {"point_base": 0, "n": system.NumPoints()}
        sl = slice(info["point_base"], info["point_base"] + info["n"])
        m = int(live[sl].sum())
        if m == 0:
            continue
        loss += float((d[sl] ** 2).sum()) / m
        grad[sl] = 2.0 * d[sl] / m
        counted += m
    return loss, grad.astype(np.float32), counted


def differentiated_rollout(system: FluidSystem, steps: int, target: np.ndarray, every: int = 1,
                           keep_tape: bool = False) -> dict:
    """Record `steps` steps from the system's current state (checkpoints every
    `every` steps), then back-propagate position_loss(target). The system is
    left at the final state; the tape is closed unless keep_tape (then the
    next rollout of the same shape reuses its storage)."""
    system.TapeBegin(steps, every)
    try:
        system.RunSteps(steps)
        order = system.TapeOrder()
        loss, dpos, counted = position_loss(system, target, order)
        gpos, gvel, gveval, gparams = system.Backward(dpos)
    finally:
        if not keep_tape:
            system.TapeEnd()
    return {"loss": loss, "points": counted, "grad_pos": gpos, "grad_vel": gvel, "grad_veval": gveval,
            "grad_params": gparams, "order": order, "dloss_dpos": dpos}


__all__ = ["PARAM_NAMES", "position_loss", "differentiated_rollout"]
