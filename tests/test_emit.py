"""The emitter's geometry (AddEmit, fluids4.0/fluid_system.cpp:336-361) on
the CPU: the lattice at emit_pos, speeds, the direction spread, COLORA."""
from __future__ import annotations

import numpy as np

from fluids3_gb300.emit import Emitter, colora


def test_emitter_lattice_speed_and_spread():
    em = Emitter(pos=(1.0, 2.0, 3.0), count=20, azimuth=30.0, tilt=60.0, speed=2.5, spread=(5.0, 4.0),
                 spacing=0.5, seed=3)
    pos, vel, clr = em.points(0.0)
    x = int(np.sqrt(20))
    k = np.arange(20)
    assert np.allclose(pos[:, 0], 1.0 + 0.5 * (k // x)) and np.allclose(pos[:, 1], 2.0 + 0.5 * (k % x))
    assert np.allclose(pos[:, 2], 3.0)
    assert np.allclose(np.linalg.norm(vel, axis=1), 2.5, rtol=1e-6)
    tilt = np.degrees(np.arccos(vel[:, 2] / 2.5))
    az = np.degrees(np.arctan2(vel[:, 1], vel[:, 0]))
    assert np.all(np.abs(tilt - 60.0) <= 4.0 + 1e-3) and np.all(np.abs(az - 30.0) <= 5.0 + 1e-3)
    assert (clr == colora(0.0, 0.0, 0.0, 1.0)).all()
    again = Emitter(pos=(1.0, 2.0, 3.0), count=20, azimuth=30.0, tilt=60.0, speed=2.5, spread=(5.0, 4.0),
                    spacing=0.5, seed=3).points(0.0)
    assert np.array_equal(again[1], vel)          # seeded


def test_colora_packs_rgba8():
    assert colora(1.0, 0.0, 0.0, 1.0) == np.uint32(0xFF0000FF)
    assert colora(0.0, 0.5, 0.0, 0.0) == np.uint32(127 << 8)
