"""Particle emitter: EmitParticles / AddEmit (fluids4.0/fluid_system.cpp:
466-472, 336-361) over fl_add_particles.

Every `every` frames the emitter adds `count` points on a sqrt(count)-wide
lattice of the given spacing at `pos`, each moving along (azimuth, tilt)
jittered by up to +-spread degrees, at `speed` -- the reference's emit_pos,
emit_rate (x: frames, y: count), emit_ang (x, y: degrees, z: speed) and
emit_spread, with a seeded generator in place of rand(). The reference's
AddEmit writes its points over indices 0..count-1 instead of the indices
AddParticle returns; here they are appended, as AddParticle intends.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .system import FluidSystem

DEG_TO_RAD = np.float32(3.14159265358979) / np.float32(180.0)


def colora(r, g, b, a) -> np.uint32:
    """COLORA (fluid_system.h:130): RGBA8 from [0,1] floats."""
    f = lambda v: np.uint32(np.float32(v) * np.float32(255.0)) & np.uint32(0xFFFFFFFF)
    return np.uint32((int(f(a)) << 24) | (int(f(b)) << 16) | (int(f(g)) << 8) | int(f(r)))


@dataclass
class Emitter:
    pos: tuple = (0.0, 0.0, 0.0)
    every: int = 1            # emit_rate.x: frames between emissions
    count: int = 0            # emit_rate.y: points per emission
    azimuth: float = 0.0      # emit_ang.x, degrees
    tilt: float = 90.0        # emit_ang.y, degrees
    speed: float = 1.0        # emit_ang.z
    spread: tuple = (0.0, 0.0)  # emit_spread.x, .y, degrees
    spacing: float = 1.0      # world units between lattice points (the reference: pdist / sim_scale)
    seed: int = 0
    frame: int = 0

    def points(self, time: float):
        """The next emission's (pos, vel, clr), AddEmit's geometry."""
        rng = np.random.default_rng((self.seed, self.frame))
        n = int(self.count)
        x = max(1, int(np.sqrt(n)))
        k = np.arange(n)
        u = rng.random((2, n)).astype(np.float32)
        ang = (u[0] * np.float32(2.0) - np.float32(1.0)) * np.float32(self.spread[0])
        tilt = (u[1] * np.float32(2.0) - np.float32(1.0)) * np.float32(self.spread[1])
        a = (np.float32(self.azimuth) + ang) * DEG_TO_RAD
        t = (np.float32(self.tilt) + tilt) * DEG_TO_RAD
        sp = np.float32(self.speed)
        vel = np.stack([np.cos(a) * np.sin(t) * sp, np.sin(a) * np.sin(t) * sp, np.cos(t) * sp], 1).astype(np.float32)
        pos = np.tile(np.asarray(self.pos, np.float32), (n, 1))
        pos[:, 0] += np.float32(self.spacing) * (k // x).astype(np.float32)
        pos[:, 1] += np.float32(self.spacing) * (k % x).astype(np.float32)
        clr = np.full(n, colora(time / 10.0, time / 5.0, time / 4.0, 1.0), np.uint32)
        return pos, vel, clr

    def step(self, system: FluidSystem) -> int:
        """EmitParticles then one Run step; returns the points added."""
        added = 0
        self.frame += 1
        if self.every > 0 and self.count > 0 and self.frame % self.every == 0:
            pos, vel, clr = self.points(system.time)
            system.AddParticles(pos, vel, vel, clr)
            added = pos.shape[0]
        system.Run()
        return added


__all__ = ["Emitter", "colora"]
