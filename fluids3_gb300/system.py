"""Host-side mirror of the reference's FluidSystem (fluids4.0/fluid_system.h:145-353)
over the C ABI. Method names and argument meaning follow the reference's
GPU pathway; every call runs the CUDA kernels of libfluids_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import call, lib
from .params import FlParams

# Buffer ids (fluids4.0/fluid.h:45-70)
FPOS, FVEL, FVEVAL, FFORCE, FPRESS, FCLR, FGCELL, FGNDX = 0, 1, 2, 3, 4, 5, 6, 7
FGRID, FGRIDCNT, FGRIDOFF = 12, 13, 14
GRID_UNDEF = 0xFFFFFFFF

_VEC3 = {FPOS, FVEL, FVEVAL, FFORCE}
_PER_CELL = {FGRIDCNT, FGRIDOFF}

PHASES = ("insert", "prefix", "sort", "pressure", "force_advance")


def default_params() -> FlParams:
    """SetupDefaultParams (fluids4.0/fluid_system.cpp:1953-2041), example-3 box."""
    p = FlParams()
    call("fl_params_default", C.byref(p))
    return p


def derive_params(p: FlParams) -> FlParams:
    """SetupSpacing/SetupGrid/FluidSetupCUDA/UpdateParamsCUDA restated in FP32."""
    out = p.copy()
    call("fl_params_derive", C.byref(out))
    return out


class PinnedArray:
    """A numpy array in page-locked host memory (fl_host_alloc)."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        ptr = C.c_void_p()
        call("fl_host_alloc", max(nbytes, 16), C.byref(ptr))
        self._ptr = ptr.value
        raw = (C.c_uint8 * max(nbytes, 16)).from_address(self._ptr)
        self.array = np.frombuffer(raw, dtype=np.uint8, count=nbytes).view(dtype).reshape(shape)

    def free(self) -> None:
        if self._ptr:
            self.array = None
            lib().fl_host_free(C.c_void_p(self._ptr))
            self._ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)


# fl_set_neighbour_passes modes, by value (FL_PASSES_*)
PASSES = ("points", "cells", "pairs", "auto")

class FluidSystem:
    """One SPH system on the current CUDA device.

    ``FluidSystem(params, max_points)`` corresponds to Initialize + Start's
    allocation (fluids4.0/fluid_system.cpp:92-168); particles are loaded with
    :meth:`SetParticles` (TransferToCUDA). ``params`` must be derived.
    """

    def __init__(self, params: FlParams, max_points: int):
        self._h = C.c_void_p()
        call("fl_create", C.byref(params), int(max_points), C.byref(self._h))
        self.max_points = int(max_points)

    @classmethod
    def batch(cls, params: list, counts: list) -> "FluidSystem":
        """Many scenes stepped together (fl_batch_create): params[k] derived,
        counts[k] points of scene k; points are passed and read back as all
        scenes' arrays concatenated in scene order."""
        self = cls.__new__(cls)
        self._h = C.c_void_p()
        arr = (FlParams * len(params))(*params)
        cnt = (C.c_int * len(counts))(*[int(c) for c in counts])
        call("fl_batch_create", arr, cnt, len(params), C.byref(self._h))
        self.max_points = int(sum(counts))
        return self

    def NumScenes(self) -> int:
        return lib().fl_num_scenes(self._h)

    def SceneInfo(self, scene: int) -> dict:
        """point_base, n, cell_base, ncells of `scene` in the concatenated layout."""
        v = [C.c_int() for _ in range(4)]
        call("fl_batch_scene_info", self._h, int(scene), *[C.byref(x) for x in v])
        return dict(point_base=v[0].value, n=v[1].value, cell_base=v[2].value, ncells=v[3].value)

    def SceneParams(self, scene: int) -> FlParams:
        p = FlParams()
        call("fl_batch_get_params", self._h, int(scene), C.byref(p))
        return p

    def SetSceneParams(self, scene: int, params: FlParams) -> None:
        """Replace one scene's physical parameters (same grid and dt)."""
        call("fl_batch_set_params", self._h, int(scene), C.byref(params))

    # -- lifetime -------------------------------------------------------------
    def close(self) -> None:
        if self._h:
            lib().fl_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # -- parameters -----------------------------------------------------------
    @property
    def params(self) -> FlParams:
        p = FlParams()
        call("fl_get_params", self._h, C.byref(p))
        return p

    def UpdateParams(self, params: FlParams) -> None:
        call("fl_set_params", self._h, C.byref(params))

    def NumPoints(self) -> int:
        return lib().fl_num_points(self._h)

    def getGridTotal(self) -> int:
        return lib().fl_grid_total(self._h)

    @property
    def time(self) -> float:
        t = C.c_float()
        call("fl_get_time", self._h, C.byref(t))
        return float(t.value)

    @time.setter
    def time(self, t: float) -> None:
        call("fl_set_time", self._h, C.c_float(t))

    # -- data -----------------------------------------------------------------
    def SetParticles(self, pos, vel=None, veval=None, force=None, press=None, clr=None) -> None:
        """TransferToCUDA (cpp:2312-2321) from (N,3) float32 / (N,) arrays."""
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        n = pos.shape[0]

        def f3(a):
            return None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(n, 3)

        def s1(a, dt):
            return None if a is None else np.ascontiguousarray(a, dtype=dt).reshape(n)

        arrs = (pos, f3(vel), f3(veval), f3(force), s1(press, np.float32), s1(clr, np.uint32))
        call("fl_set_particles", self._h, n, *[_ptr(a) for a in arrs])

    def GetBuffer(self, buf_id: int) -> np.ndarray:
        """Read buffer ``buf_id`` back in fluid.h layout."""
        n = self.getGridTotal() if buf_id in _PER_CELL else self.NumPoints()
        if buf_id in _VEC3:
            out = np.empty((n, 3), dtype=np.float32)
        elif buf_id == FPRESS:
            out = np.empty(n, dtype=np.float32)
        else:
            out = np.empty(n, dtype=np.uint32)
        if n:
            call("fl_get_buffer", self._h, int(buf_id), _ptr(out), out.nbytes)
        return out

    def state(self) -> dict:
        """All per-point buffers and the grid, as numpy arrays."""
        names = {FPOS: "pos", FVEL: "vel", FVEVAL: "veval", FFORCE: "force", FPRESS: "press",
                 FCLR: "clr", FGCELL: "gcell", FGNDX: "gndx", FGRIDCNT: "gridcnt",
                 FGRIDOFF: "gridoff"}
        return {v: self.GetBuffer(k) for k, v in names.items()}

    def AddParticles(self, pos, vel=None, veval=None, clr=None) -> None:
        """AddParticle (cpp:274-290) for every row of pos (N,3): appended
        after the live points."""
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        k = pos.shape[0]
        f3 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(k, 3)
        c = None if clr is None else np.ascontiguousarray(clr, dtype=np.uint32).reshape(k)
        call("fl_add_particles", self._h, k, *[_ptr(a) for a in (pos, f3(vel), f3(veval), c)])

    def SavePoints(self, path, with_veval: bool = True) -> None:
        """SavePoints (cpp:1511-1545): the points to a .pts file; with_veval
        adds the evaluated velocity for an exact resume."""
        call("fl_save_points", self._h, str(path).encode(), 1 if with_veval else 0)

    def LoadPoints(self, path) -> None:
        """RunPlayback (cpp:1787-1841): the points of a .pts file."""
        call("fl_load_points", self._h, str(path).encode())

    def SampleParticles(self, res, bmin, bmax, scalar: float = 1.0 / 100.0, sort_first: bool = True,
                        out=None):
        """SampleParticlesCUDA (cpp:2497-2507): Gaussian-weighted particle
        density on a res = (x, y, z) voxel lattice over [bmin, bmax); returns
        (or fills `out`, host array or device pointer) shape (z, y, x)."""
        r = (C.c_int * 3)(*[int(v) for v in res])
        lo = (C.c_float * 3)(*[float(v) for v in bmin])
        hi = (C.c_float * 3)(*[float(v) for v in bmax])
        if out is None or isinstance(out, np.ndarray):
            arr = out if out is not None else np.empty((int(res[2]), int(res[1]), int(res[0])), np.float32)
            call("fl_sample_volume", self._h, _ptr(arr), r, lo, hi, C.c_float(scalar), 1 if sort_first else 0)
            return arr
        call("fl_sample_volume", self._h, out, r, lo, hi, C.c_float(scalar), 1 if sort_first else 0)
        return None

    # -- phases (fluid_system.h:249-256) --------------------------------------
    def InsertParticlesCUDA(self, readback: bool = False):
        n, c = self.NumPoints(), self.getGridTotal()
        if not readback:
            call("fl_insert_particles", self._h, None, None, None)
            return None
        gcell = np.empty(n, np.uint32)
        gndx = np.empty(n, np.uint32)
        gcnt = np.empty(c, np.uint32)
        call("fl_insert_particles", self._h, _ptr(gcell), _ptr(gndx), _ptr(gcnt))
        return gcell, gndx, gcnt

    def PrefixSumCellsCUDA(self, zero_offsets: int = 1, readback: bool = False):
        if not readback:
            call("fl_prefix_sum_cells", self._h, None, int(zero_offsets))
            return None
        goff = np.empty(self.getGridTotal(), np.uint32)
        call("fl_prefix_sum_cells", self._h, _ptr(goff), int(zero_offsets))
        return goff

    def CountingSortFullCUDA(self, readback: bool = False):
        if not readback:
            call("fl_counting_sort_full", self._h, None)
            return None
        ppos = np.empty((self.NumPoints(), 3), np.float32)
        call("fl_counting_sort_full", self._h, _ptr(ppos))
        return ppos

    def ComputePressureCUDA(self) -> None:
        call("fl_compute_pressure", self._h)

    def ComputeForceCUDA(self) -> None:
        call("fl_compute_force", self._h)

    def AdvanceCUDA(self, time: float, dt: float, ss: float) -> None:
        call("fl_advance", self._h, C.c_float(time), C.c_float(dt), C.c_float(ss))

    def Run(self) -> None:
        """One RUN_GPU_FULL step (cpp:506-524) on the fused kernels, then time += dt."""
        call("fl_run", self._h)

    def RunFromHost(self, pos, vel=None, veval=None, clr=None, pos_out=None) -> None:
        """TransferToCUDA + Run (+ the new positions into pos_out, an (N,3)
        float32 array) in one call (fl_run_from_host); equal to SetParticles
        + Run (+ GetBuffer(FPOS)). Arrays in page-locked memory (PinnedArray)
        let the uploads of everything but the positions overlap the step's
        first kernels and the readback overlap its force pass."""
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        n = pos.shape[0]

        def f3(a):
            return None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(n, 3)

        c = None if clr is None else np.ascontiguousarray(clr, dtype=np.uint32).reshape(n)
        if pos_out is not None and (pos_out.dtype != np.float32 or pos_out.shape != (n, 3)
                                    or not pos_out.flags.c_contiguous):
            raise ValueError("pos_out must be a C-contiguous (N, 3) float32 array")
        arrs = (pos, f3(vel), f3(veval), c, pos_out)
        call("fl_run_from_host", self._h, n, *[_ptr(a) for a in arrs])

    def RunSteps(self, nsteps: int) -> None:
        """``nsteps`` Run steps replayed from a captured CUDA graph."""
        call("fl_run_steps", self._h, int(nsteps))

    def SaveCheckpoint(self, slot: int = 0) -> None:
        call("fl_checkpoint_save", self._h, int(slot))

    def RestoreCheckpoint(self, slot: int = 0) -> None:
        call("fl_checkpoint_restore", self._h, int(slot))

    def Sync(self) -> None:
        call("fl_sync", self._h)

    def DeviceStatus(self) -> int:
        v = C.c_uint32()
        call("fl_device_status", self._h, C.byref(v))
        return int(v.value)

    def IntegrityCheck(self) -> int:
        """IntegrityCheck (cpp:2426-2453): number of inconsistent sorted slots."""
        bad = C.c_int64()
        call("fl_integrity_check", self._h, C.byref(bad))
        return int(bad.value)

    # -- adjoint (no counterpart in the reference) ----------------------------
    def TapeBegin(self, max_steps: int, every: int = 1, keep_lists: bool = False) -> None:
        """Record the Run steps that follow (up to ``max_steps``; a checkpoint of
        the state every ``every`` steps) for Backward. keep_lists: segment
        replays keep their pair lists (more memory, faster reverse steps)."""
        call("fl_tape_begin_ex", self._h, int(max_steps), int(every), 1 if keep_lists else 0)

    def TapeSteps(self) -> int:
        return int(lib().fl_tape_steps(self._h))

    def TapeOrder(self) -> np.ndarray:
        """Per current slot, the point's index when recording began."""
        out = np.empty(self.NumPoints(), np.uint32)
        if out.size:
            call("fl_tape_order", self._h, _ptr(out))
        return out

    def BackwardScaled(self, dpos=None, dvel=None, dveval=None):
        """Backward for long rollouts (fl_backward_scaled): returns (gpos,
        gvel, gveval, gparams, exponents) with the state gradients as
        mantissas; the gradient of scene k is mantissa * 2**exponents[k]."""
        n = self.NumPoints()
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float32).reshape(n, 3)
                for a in (dpos, dvel, dveval)]
        outs = [np.empty((n, 3), np.float32) for _ in range(3)]
        gp = np.zeros((self.NumScenes(), 3), np.float64)
        ex = np.zeros(self.NumScenes(), np.int32)
        call("fl_backward_scaled", self._h, *[_ptr(a) for a in keep], *[_ptr(o) for o in outs], _ptr(gp), _ptr(ex))
        return outs[0], outs[1], outs[2], gp, ex

    def Backward(self, dpos=None, dvel=None, dveval=None, want_state: bool = True):
        """Reverse pass over the recorded steps. ``d*``: dL/d(final pos, vel,
        veval) as (N,3) arrays in the current slot order (None = zero), or device
        pointers (int). Returns (gpos, gvel, gveval, gparams): dL/d(initial
        state) in the order of the recording's start, and per scene
        dL/d(pvisc, prest_dens, pintstiff) as an (nscenes, 3) float64 array."""
        n = self.NumPoints()

        def arg(a):
            if a is None or isinstance(a, int):
                return a
            a = np.ascontiguousarray(a, dtype=np.float32).reshape(n, 3)
            keep.append(a)
            return _ptr(a)

        keep: list = []
        outs = [np.empty((n, 3), np.float32) for _ in range(3)] if want_state else [None] * 3
        gp = np.zeros((self.NumScenes(), 3), np.float64)
        call("fl_backward", self._h, arg(dpos), arg(dvel), arg(dveval), *[_ptr(o) for o in outs], _ptr(gp))
        return outs[0], outs[1], outs[2], gp

    def TapeEnd(self) -> None:
        call("fl_tape_end", self._h)

    CONSERVATION = ("count", "mass", "px", "py", "pz", "kinetic", "potential", "sx", "sy", "sz")

    def Conservation(self) -> np.ndarray:
        """(nscenes, 10) FP64 sums: count, mass, momentum, kinetic and
        potential energy, sum of positions (fl_conservation)."""
        out = np.zeros((self.NumScenes(), 10), np.float64)
        call("fl_conservation", self._h, _ptr(out))
        return out

    def Autotune(self, steps: int = 3) -> dict:
        """Pick the fastest launch shapes for this system's work (state kept)."""
        call("fl_autotune", self._h, int(steps), None)
        return self.LaunchShapes()

    def LaunchShapes(self) -> dict:
        """Threads per block of the density, force and sort passes and cell
        entries per warp of the cell sort."""
        out = (C.c_int * 4)()
        call("fl_launch_shapes", self._h, out)
        return {"density": out[0], "force": out[1], "sort": out[2], "sort_cells": out[3]}

    def SetLaunchShapes(self, density: int = 0, force: int = 0, sort: int = 0, sort_cells: int = 0) -> None:
        """Pin the launch shapes (0: compiled default), e.g. from LaunchShapes()
        after an Autotune in an earlier run."""
        shapes = (C.c_int * 4)(int(density), int(force), int(sort), int(sort_cells))
        call("fl_set_launch_shapes", self._h, shapes)

    def SetNeighbourPasses(self, mode: str) -> None:
        """Neighbour passes of the fused step: "points", one thread per point
        (the reference's loop structure); "cells", one warp per 64 points of
        a cell walks their shared search block in lockstep; "pairs", the
        per-point passes with a density walk shared by two points of a cell
        that visit the same candidates (every density pass of the system);
        "auto" (default), "points" until the largest cell reaches 512
        points, "cells" from then until it falls below 384. Results are
        bit-identical."""
        call("fl_set_neighbour_passes", self._h, PASSES.index(mode))

    def NeighbourPasses(self) -> str:
        return PASSES[call("fl_neighbour_passes", self._h)]

    def NeighbourPassesInUse(self) -> str:
        """The passes the next fused step takes ("auto" resolved)."""
        return PASSES[call("fl_neighbour_passes_in_use", self._h)]

    def PassesSteps(self) -> tuple:
        """Fused steps issued so far with the per-point passes and with the
        cell tasks."""
        c = (C.c_int64 * 2)()
        call("fl_passes_steps", self._h, c)
        return int(c[0]), int(c[1])

    # -- timing ---------------------------------------------------------------
    def SetTiming(self, enable: bool) -> None:
        call("fl_set_timing", self._h, 1 if enable else 0)

    def TimeSteps(self, nsteps: int, graph: bool = True, restart_every: int = 0,
                  restart_slot: int = 0) -> float:
        """Device milliseconds for ``nsteps`` Run steps between CUDA events on the
        system stream; with ``restart_every`` the steps run as segments that each
        restart from checkpoint ``restart_slot`` (restores inside the interval)."""
        ms = C.c_double()
        call("fl_time_steps", self._h, int(nsteps), 1 if graph else 0, int(restart_every),
             int(restart_slot), C.byref(ms))
        return float(ms.value)

    def PhaseTimes(self) -> tuple[dict, int]:
        ms = (C.c_double * 8)()
        steps = C.c_int()
        call("fl_get_phase_times", self._h, ms, C.byref(steps))
        names = ("insert", "scan", "scatter", "sort", "density", "force_advance")
        return {k: float(ms[i]) for i, k in enumerate(names)}, int(steps.value)

    def stream(self) -> int:
        return int(lib().fl_stream(self._h) or 0)


__all__ = ["FluidSystem", "PinnedArray", "default_params", "derive_params", "FPOS", "FVEL", "FVEVAL",
           "FFORCE", "FPRESS", "FCLR", "FGCELL", "FGNDX", "FGRID", "FGRIDCNT", "FGRIDOFF",
           "GRID_UNDEF", "_lib"]
