"""Parameter block of the SPH step: a ctypes mirror of ``fl_params``
(include/fluids_gb300.h), whose names follow the reference's FParams
(fluids4.0/fluid.h:155-192)."""
from __future__ import annotations

import ctypes as C

F3 = C.c_float * 3
I3 = C.c_int * 3


class FlParams(C.Structure):
    _fields_ = [
        # inputs
        ("sim_scale", C.c_float), ("pvisc", C.c_float), ("prest_dens", C.c_float),
        ("pmass", C.c_float), ("pradius", C.c_float), ("psmoothradius", C.c_float),
        ("pintstiff", C.c_float), ("bound_stiff", C.c_float), ("bound_damp", C.c_float),
        ("bound_slope", C.c_float), ("bound_friction", C.c_float),
        ("bound_wall_force", C.c_float), ("bound_wall_freq", C.c_float),
        ("AL", C.c_float), ("VL", C.c_float), ("grav_dir", F3), ("grav_amt", C.c_float),
        ("bound_min", F3), ("bound_max", F3), ("grid_density", C.c_float), ("dt", C.c_float),
        # derived
        ("grid_size", C.c_float), ("r2", C.c_float), ("d2", C.c_float), ("rd2", C.c_float),
        ("poly6kern", C.c_float), ("spikykern", C.c_float), ("lapkern", C.c_float),
        ("vterm", C.c_float), ("AL2", C.c_float), ("VL2", C.c_float), ("gravity", F3),
        ("pdist", C.c_float), ("gridMin", F3), ("gridMax", F3), ("gridSize", F3),
        ("gridDelta", F3), ("gridRes", I3), ("gridScanMax", I3), ("gridSrch", C.c_int),
        ("gridTotal", C.c_int), ("gridAdjCnt", C.c_int), ("gridAdj", C.c_int * 216),
    ]

    INPUTS = ("sim_scale", "pvisc", "prest_dens", "pmass", "pradius", "psmoothradius",
              "pintstiff", "bound_stiff", "bound_damp", "bound_slope", "bound_friction",
              "bound_wall_force", "bound_wall_freq", "AL", "VL", "grav_dir", "grav_amt",
              "bound_min", "bound_max", "grid_density", "dt")

    def copy(self) -> "FlParams":
        out = FlParams()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(FlParams))
        return out

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if not isinstance(v, (int, float)) else v
        return d

    def set(self, **kw) -> "FlParams":
        for k, v in kw.items():
            if k not in dict(self._fields_):
                raise KeyError(f"unknown parameter {k!r}")
            if isinstance(v, (list, tuple)):
                arr = getattr(self, k)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(self, k, v)
        return self
