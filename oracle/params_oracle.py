"""TEST INFRASTRUCTURE ONLY: an independent numpy-float32 restatement of the
reference's host parameter derivation, used to check fl_params_derive.

Follows fluids4.0/fluid_system.cpp line by line:
  SetupSpacing (grid part)  2101, 2114-2116
  SetupGrid                 793-846
  FluidSetupCUDA            2249-2287 (scan limits, adjacency)
  UpdateParamsCUDA          2289-2310
numpy float32 scalar arithmetic rounds every operation to float32 (no
fusion); the two products upstream writes with double literals (1.5 * h,
2.0 * cell) are formed in float64 and rounded, as C++ does.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

f32 = np.float32

# The reference calls the C library's powf (pow(float, float) in C++); use
# the same routine so the restatement rounds identically on this machine.
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.powf.restype = ctypes.c_float
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]


def powf(x, y) -> np.float32:
    return f32(_libm.powf(float(x), float(y)))


def derive(inp: dict) -> dict:
    ss = f32(inp["sim_scale"])
    h = f32(inp["psmoothradius"])
    gd = f32(inp["grid_density"])
    out = {}
    grid_size = f32(1.5 * float(h) / float(gd))
    out["grid_size"] = grid_size
    border = f32(2.0 * float(f32(grid_size / ss)))
    gmin = [f32(inp["bound_min"][k]) - border for k in range(3)]
    gmax = [f32(inp["bound_max"][k]) + border for k in range(3)]
    out["gridMin"], out["gridMax"] = gmin, gmax
    wcell = f32(grid_size / ss)
    res, size = [], []
    for k in range(3):
        span = f32(gmax[k] - gmin[k])
        r = int(np.ceil(f32(span / wcell)))
        res.append(r)
        size.append(f32(f32(f32(r) * grid_size) / ss))
    out["gridRes"], out["gridSize"] = res, size
    out["gridDelta"] = [f32(f32(res[k]) / size[k]) for k in range(3)]
    out["gridTotal"] = res[0] * res[1] * res[2]
    srch = int(f32(np.floor(f32(f32(f32(2.0) * f32(h / ss)) / wcell)) + f32(1.0)))
    srch = max(srch, 2)
    out["gridSrch"] = srch
    out["gridAdjCnt"] = srch ** 3
    out["gridScanMax"] = [r - srch for r in res]
    out["gridAdj"] = [(y * res[2] + z) * res[0] + x
                      for y in range(srch) for z in range(srch) for x in range(srch)]
    out["gravity"] = [f32(f32(inp["grav_dir"][k]) * f32(inp["grav_amt"])) for k in range(3)]
    out["AL2"] = f32(f32(inp["AL"]) * f32(inp["AL"]))
    out["VL2"] = f32(f32(inp["VL"]) * f32(inp["VL"]))
    r2 = f32(h * h)
    out["r2"] = r2
    pi = f32(3.141592)
    out["poly6kern"] = f32(f32(315.0) / f32(f32(f32(64.0) * pi) * powf(h, 9.0)))
    out["spikykern"] = f32(f32(-45.0) / f32(pi * powf(h, 6.0)))
    out["lapkern"] = f32(f32(45.0) / f32(pi * powf(h, 6.0)))
    d2 = f32(ss * ss)
    out["d2"] = d2
    out["rd2"] = f32(r2 / d2)
    out["vterm"] = f32(out["lapkern"] * f32(inp["pvisc"]))
    return out


def derive_flparams(p):
    """A copy of the FlParams block `p` (inputs set) with every derived field
    filled by derive() above -- fl_params_derive never runs, so a caller
    that must stay independent of the product library (the reference arm of
    the benchmark) gets its parameters from this restatement alone."""
    out = p.copy()
    inp = {k: (list(getattr(p, k)) if not isinstance(getattr(p, k), (int, float)) else getattr(p, k))
           for k in ("sim_scale", "psmoothradius", "grid_density", "bound_min", "bound_max", "grav_dir",
                     "grav_amt", "AL", "VL", "pvisc")}
    for k, v in derive(inp).items():
        if isinstance(v, list):
            out.set(**{k: [int(x) if isinstance(x, int) else float(x) for x in v]})
        else:
            out.set(**{k: int(v) if isinstance(v, int) else float(v)})
    # UpdateParamsCUDA's rest spacing (cpp:2300): powf(mass / rest density, 1/3)
    out.pdist = float(powf(f32(f32(p.pmass) / f32(p.prest_dens)), f32(1.0) / f32(3.0)))
    return out


def compare(lib_params, tol_ulps: int = 0) -> list[str]:
    """Fields where fl_params_derive's result differs from this restatement.
    The powf-based kernels (poly6/spiky/lap) are compared within `tol_ulps`
    units in the last place (0 on one machine; libm builds may differ)."""
    inp = {k: (list(getattr(lib_params, k)) if not isinstance(getattr(lib_params, k), (int, float))
               else getattr(lib_params, k)) for k in
           ("sim_scale", "psmoothradius", "grid_density", "bound_min", "bound_max", "grav_dir",
            "grav_amt", "AL", "VL", "pvisc")}
    want = derive(inp)
    bad = []
    for k, v in want.items():
        got = getattr(lib_params, k)
        if k == "gridAdj":
            got = list(got)[: len(v)]
        elif not isinstance(got, (int, float)):
            got = list(got)
        gv = np.asarray(got, dtype=np.asarray(v).dtype if not isinstance(v, list) or not isinstance(v[0], int) else np.int64)
        wv = np.asarray(v, dtype=gv.dtype)
        if k in ("poly6kern", "spikykern", "lapkern"):
            ulp = abs(int(np.float32(got).view(np.int32)) - int(np.float32(v).view(np.int32)))
            if ulp > tol_ulps:
                bad.append(f"{k}: {got} vs {v} ({ulp} ulp)")
        elif not np.array_equal(gv, wv):
            bad.append(f"{k}: {got} vs {v}")
    return bad


def spacing_check() -> bool:
    return math.isclose(float(f32(0.0059) / f32(0.004)), 1.475, rel_tol=1e-6)
