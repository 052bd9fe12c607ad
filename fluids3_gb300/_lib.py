"""Loads the in-tree CUDA library libfluids_gb300.so and declares the C ABI.

There is no fallback: if the library is missing or fails to load, every
entry point raises. Build it with ``python -m fluids3_gb300.build`` (or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from .params import FlParams

LIB_PATH = Path(__file__).resolve().parent / "libfluids_gb300.so"

_lock = threading.Lock()
_lib = None

u32p = C.POINTER(C.c_uint32)
f32p = C.POINTER(C.c_float)
vp = C.c_void_p

# (name, restype, argtypes) for every symbol declared in include/fluids_gb300.h
SIGNATURES = [
    ("fl_params_default", C.c_int, [C.POINTER(FlParams)]),
    ("fl_params_derive", C.c_int, [C.POINTER(FlParams)]),
    ("fl_create", C.c_int, [C.POINTER(FlParams), C.c_int, C.POINTER(vp)]),
    ("fl_destroy", C.c_int, [vp]),
    ("fl_batch_create", C.c_int, [C.POINTER(FlParams), C.POINTER(C.c_int), C.c_int, C.POINTER(vp)]),
    ("fl_num_scenes", C.c_int, [vp]),
    ("fl_batch_scene_info", C.c_int, [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("fl_set_params", C.c_int, [vp, C.POINTER(FlParams)]),
    ("fl_get_params", C.c_int, [vp, C.POINTER(FlParams)]),
    ("fl_num_points", C.c_int, [vp]),
    ("fl_grid_total", C.c_int, [vp]),
    ("fl_get_time", C.c_int, [vp, f32p]),
    ("fl_set_time", C.c_int, [vp, C.c_float]),
    ("fl_set_particles", C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, vp]),
    ("fl_get_buffer", C.c_int, [vp, C.c_int, vp, C.c_size_t]),
    ("fl_host_alloc", C.c_int, [C.c_size_t, C.POINTER(vp)]),
    ("fl_host_free", C.c_int, [vp]),
    ("fl_export_device", C.c_int, [vp, C.c_int, vp, C.c_size_t]),
    ("fl_import_device", C.c_int, [vp, C.c_int, vp, vp, vp]),
    ("fl_insert_particles", C.c_int, [vp, vp, vp, vp]),
    ("fl_prefix_sum_cells", C.c_int, [vp, vp, C.c_int]),
    ("fl_counting_sort_full", C.c_int, [vp, vp]),
    ("fl_compute_pressure", C.c_int, [vp]),
    ("fl_compute_force", C.c_int, [vp]),
    ("fl_advance", C.c_int, [vp, C.c_float, C.c_float, C.c_float]),
    ("fl_run", C.c_int, [vp]),
    ("fl_run_from_host", C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp]),
    ("fl_run_steps", C.c_int, [vp, C.c_int]),
    ("fl_checkpoint_save", C.c_int, [vp, C.c_int]),
    ("fl_checkpoint_restore", C.c_int, [vp, C.c_int]),
    ("fl_sync", C.c_int, [vp]),
    ("fl_device_status", C.c_int, [vp, u32p]),
    ("fl_integrity_check", C.c_int, [vp, C.POINTER(C.c_int64)]),
    ("fl_set_timing", C.c_int, [vp, C.c_int]),
    ("fl_time_steps", C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    ("fl_get_phase_times", C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    ("fl_prefix_sum_noalloc", C.c_int, [vp, vp, C.c_int, C.c_int, vp, vp]),
    ("fl_test_scan_timeout", C.c_int, [vp, C.c_int]),
    ("fl_test_scan_noalloc_timeout", C.c_int, [vp, vp, C.c_int, vp, C.c_int, vp]),
    ("fl_set_reverse_lists", C.c_int, [vp, C.c_int]),
    ("fl_neighbour_passes_in_use", C.c_int, [vp]),
    ("fl_passes_steps", C.c_int, [vp, C.POINTER(C.c_int64)]),
    ("fl_batch_get_params", C.c_int, [vp, C.c_int, C.POINTER(FlParams)]),
    ("fl_batch_set_params", C.c_int, [vp, C.c_int, C.POINTER(FlParams)]),
    ("fl_add_particles", C.c_int, [vp, C.c_int, vp, vp, vp, vp]),
    ("fl_autotune", C.c_int, [vp, C.c_int, vp]),
    ("fl_launch_shapes", C.c_int, [vp, vp]),
    ("fl_set_neighbour_passes", C.c_int, [vp, C.c_int]),
    ("fl_neighbour_passes", C.c_int, [vp]),
    ("fl_set_launch_shapes", C.c_int, [vp, vp]),
    ("fl_conservation", C.c_int, [vp, vp]),
    ("fl_pts_write", C.c_int, [C.c_char_p, C.c_int, vp, vp, vp, vp]),
    ("fl_pts_read", C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), vp, vp, vp, vp]),
    ("fl_save_points", C.c_int, [vp, C.c_char_p, C.c_int]),
    ("fl_load_points", C.c_int, [vp, C.c_char_p]),
    ("fl_sample_volume", C.c_int, [vp, vp, C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.c_float, C.c_int]),
    ("fl_tape_begin", C.c_int, [vp, C.c_int, C.c_int]),
    ("fl_tape_begin_ex", C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
    ("fl_tape_steps", C.c_int, [vp]),
    ("fl_tape_order", C.c_int, [vp, vp]),
    ("fl_backward", C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp]),
    ("fl_backward_scaled", C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("fl_tape_end", C.c_int, [vp]),
    ("fl_stream", vp, [vp]),
    ("fl_last_error", C.c_char_p, []),
    ("fl_abi_version", C.c_int, []),
]


class FluidsError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, call: str, code: int, message: str):
        super().__init__(f"{call} failed ({code}): {message}")
        self.call = call
        self.code = code


def lib():
    """The loaded library (loads on first use; raises if it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise ImportError(
                    f"{LIB_PATH.name} is not built; run `python -m fluids3_gb300.build` "
                    "(nvcc for sm_103a) -- there is no CPU fallback")
            handle = C.CDLL(str(LIB_PATH))
            for name, res, args in SIGNATURES:
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def check(call: str, code: int) -> int:
    if code < 0:
        msg = lib().fl_last_error()
        raise FluidsError(call, code, msg.decode() if msg else "")
    return code


def call(name: str, *args) -> int:
    return check(name, getattr(lib(), name)(*args))
