"""Batched parameter fit by adjoint gradient descent (no counterpart in the
reference).

Many scenes step together in one batched system. Each scene's target is the
trajectory of a run with that scene's hidden parameters; the fit recovers
per-scene viscosity and IntStiff from a common starting guess by Adam steps
on adjoint gradients.

The loss follows the target trajectory in windows (multiple shooting): each
window starts from the target state at its first step, runs `window` steps
with the current parameters and compares the positions to the target's at
its last step. Matching a whole 100-step trajectory from its first state in
one rollout does not work for this system: particle trajectories diverge
exponentially (the step's Jacobian grows gradients by about 1.3-1.5x per
step), so the exact gradient of a 100-step loss is of order 1e15 and points
nowhere useful, while over a 10-20 step window it is informative.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import scenes as S
from .rollout import differentiated_rollout
from .system import FGCELL, FPOS, FVEL, FVEVAL, GRID_UNDEF, FluidSystem, derive_params


@dataclass
class FitResult:
    hidden_visc: np.ndarray
    visc: np.ndarray
    stiff: np.ndarray
    losses: list = field(default_factory=list)

    @property
    def visc_rel_err(self) -> np.ndarray:
        return np.abs(self.visc - self.hidden_visc) / self.hidden_visc


@dataclass
class Trajectory:
    """Per window boundary b: the state of every point (indexed by its
    initial order; out-of-range points keep their parked values), whether it
    was inside the scan range, and the time."""
    pos: list
    vel: list
    veval: list
    valid: list
    time: list


def set_scene_physics(system: FluidSystem, scene: int, visc: float, stiff: float) -> None:
    p = system.SceneParams(scene)
    p.pvisc = float(visc)
    p.pintstiff = float(stiff)
    system.SetSceneParams(scene, derive_params(p))


def record_trajectory(system: FluidSystem, steps: int, window: int) -> Trajectory:
    """Run `steps` steps from checkpoint 0 and keep the state at every
    multiple of `window` steps (0 included), indexed by initial order."""
    n = system.NumPoints()
    system.RestoreCheckpoint(0)
    tr = Trajectory([], [], [], [], [])
    system.TapeBegin(steps, steps)             # for the identity map only
    for b in range(steps // window + 1):
        if b:
            system.RunSteps(window)
        order = system.TapeOrder()
        live = system.GetBuffer(FGCELL) != GRID_UNDEF if b else np.ones(n, bool)
        for lst, buf in ((tr.pos, FPOS), (tr.vel, FVEL), (tr.veval, FVEVAL)):
            a = np.empty((n, 3), np.float32)
            a[order] = system.GetBuffer(buf)
            lst.append(a)
        v = np.empty(n, bool)
        v[order] = live
        tr.valid.append(v)
        tr.time.append(system.time)
    system.TapeEnd()
    return tr


def window_loss_gradient(system: FluidSystem, tr: Trajectory, b: int, window: int, every: int):
    """One window from boundary b: start at the target state, run `window`
    steps, loss against the target positions at boundary b + 1."""
    system.SetParticles(tr.pos[b], tr.vel[b], tr.veval[b])
    system.time = tr.time[b]
    target = np.where(tr.valid[b + 1][:, None], tr.pos[b + 1].astype(np.float64), np.nan)
    return differentiated_rollout(system, window, target, every, keep_tape=True)


def batched_fit(scs: list, steps: int = 100, window: int = 10, every: int = 10, iters: int = 30,
                lr: float = 0.05, start=(0.3, 1.0), log=None) -> FitResult:
    """Fit per-scene (viscosity, IntStiff) of `scs` (hidden viscosity in
    params.pvisc) from `start`: Adam on the parameters relative to `start`,
    each iteration summing the gradients of all steps // window windows."""
    hidden = np.array([sc.params.pvisc for sc in scs], np.float64)
    cat = S.concat(scs)
    k = len(scs)
    with FluidSystem.batch([sc.params for sc in scs], [sc.n for sc in scs]) as b:
        b.SetParticles(cat["pos"], cat["vel"], cat["veval"], clr=cat["clr"])
        b.SaveCheckpoint(0)
        tr = record_trajectory(b, steps, window)
        scale = np.array(start, np.float64)
        u = np.ones((k, 2))                    # parameters / start
        m = np.zeros((k, 2)); v = np.zeros((k, 2))
        b1, b2, eps = 0.9, 0.999, 1e-12
        res = FitResult(hidden_visc=hidden, visc=u[:, 0] * scale[0], stiff=u[:, 1] * scale[1])
        for it in range(iters):
            for sc in range(k):
                set_scene_physics(b, sc, u[sc, 0] * scale[0], u[sc, 1] * scale[1])
            g = np.zeros((k, 2))
            loss = 0.0
            for w in range(steps // window):
                r = window_loss_gradient(b, tr, w, window, every)
                gw = r["grad_params"][:, [0, 2]] * scale          # d loss / d u
                # a pair at near-zero distance can overflow a scene's window
                # gradient (its derivative is genuinely unbounded): skip it
                ok = np.isfinite(gw).all(axis=1)
                g[ok] += gw[ok]
                loss += r["loss"]
            m = b1 * m + (1 - b1) * g
            v = b2 * v + (1 - b2) * g * g
            mh = m / (1 - b1 ** (it + 1)); vh = v / (1 - b2 ** (it + 1))
            u = np.clip(u - lr * mh / (np.sqrt(vh) + eps), 0.05, 5.0)
            res.losses.append(loss)
            if log:
                log(it, loss, u[:, 0] * scale[0])
        b.TapeEnd()
        res.visc = u[:, 0] * scale[0]
        res.stiff = u[:, 1] * scale[1]
    return res


__all__ = ["FitResult", "Trajectory", "batched_fit", "record_trajectory", "set_scene_physics",
           "window_loss_gradient"]
