"""The scan's bounded look-back wait, made to run out on purpose.

The cell scan is the library's only device-side wait (a CTA polls its
predecessor tiles' descriptors). Every poll loop has an iteration limit,
after which the kernel records FL_DEV_SPIN_TIMEOUT in the device error word
and returns, so a lost predecessor never hangs the GPU. Here the test hook
fl_test_scan_timeout withholds tile 0 -- one CTA fewer, the tile ticket
starting at 1, every index in bounds -- with a 256-poll limit: tile 1's
wait for tile 0 cannot end by itself. The call must return, fl_sync must
report FL_ERR_DEVICE with the timeout flag, and the system must step
normally afterwards.
"""
from __future__ import annotations

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import _lib, scenes
from oracle import oracle as O

from helpers import FIELDS, assert_bit_equal

pytestmark = pytest.mark.gpu

FL_ERR_DEVICE = -5
FL_DEV_SPIN_TIMEOUT = 0x1


def test_system_scan_wait_runs_out_and_is_reported():
    sc = scenes.wave_tank(n=60_000)
    p = sc.params
    assert p.gridTotal + 1 > 2 * 4096          # at least two scan tiles
    lib = _lib.lib()
    with F.FluidSystem(p, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        s.InsertParticlesCUDA()
        assert lib.fl_test_scan_timeout(s.handle, 256) == 0, lib.fl_last_error()
        flags = np.zeros(1, np.uint32)
        assert lib.fl_device_status(s.handle, flags.ctypes.data_as(_lib.u32p)) == 0
        assert flags[0] & FL_DEV_SPIN_TIMEOUT
        assert lib.fl_sync(s.handle) == FL_ERR_DEVICE
        assert b"timed out" in lib.fl_last_error()
        # the error word is cleared and the context is intact: a full step
        # from the same inputs matches the oracle bit for bit
        assert lib.fl_sync(s.handle) == 0
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        s.Run()
        s.Sync()
        st = s.state()
    ref = O.State.new(p, sc.pos, sc.vel, sc.veval, sc.clr)
    O.step(p, ref, 0.0, threads=8)
    for k in ("gcell", "gndx", "press", "force"):
        assert_bit_equal(st[k], getattr(ref, k), k)
    assert set(FIELDS) <= set(st)
