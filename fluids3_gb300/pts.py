"""The .pts point-file format of the reference's SavePoints / RunPlayback
(fluids4.0/fluid_system.cpp:1511-1545, 1787-1841), through the C ABI
(fl_pts_write / fl_pts_read). See include/fluids_gb300.h for the layout."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import call


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def write_pts(path, pos, vel, clr, veval=None) -> None:
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    vel = np.ascontiguousarray(vel, np.float32).reshape(n, 3)
    clr = np.ascontiguousarray(clr, np.uint32).reshape(n)
    ve = None if veval is None else np.ascontiguousarray(veval, np.float32).reshape(n, 3)
    call("fl_pts_write", str(path).encode(), n, _ptr(pos), _ptr(vel), _ptr(clr), _ptr(ve))


def read_pts(path) -> dict:
    """{pos, vel, clr, veval (None without the fourth field), nfields}."""
    n, nf = C.c_int(), C.c_int()
    call("fl_pts_read", str(path).encode(), C.byref(n), C.byref(nf), None, None, None, None)
    k = n.value
    pos, vel, ve = (np.empty((k, 3), np.float32) for _ in range(3))
    clr = np.empty(k, np.uint32)
    call("fl_pts_read", str(path).encode(), C.byref(n), C.byref(nf), _ptr(pos), _ptr(vel), _ptr(clr), _ptr(ve))
    return {"pos": pos, "vel": vel, "clr": clr, "veval": ve if nf.value >= 4 else None, "nfields": nf.value}


__all__ = ["write_pts", "read_pts"]
