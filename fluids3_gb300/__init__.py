"""GB300-native (sm_103a) SPH time step with the reference FluidSystem's call surface.

The compute path is libfluids_gb300.so (hand-written CUDA + a C ABI,
include/fluids_gb300.h); this package is its Python host mirror.
"""
from .params import FlParams
from .system import (FCLR, FFORCE, FGCELL, FGNDX, FGRID, FGRIDCNT, FGRIDOFF, FPOS, FPRESS,
                     FVEL, FVEVAL, GRID_UNDEF, FluidSystem, PinnedArray, default_params,
                     derive_params)
from ._lib import FluidsError, LIB_PATH, lib

__all__ = ["FlParams", "FluidSystem", "PinnedArray", "FluidsError", "default_params", "derive_params", "lib",
           "LIB_PATH", "FPOS", "FVEL", "FVEVAL", "FFORCE", "FPRESS", "FCLR", "FGCELL", "FGNDX",
           "FGRID", "FGRIDCNT", "FGRIDOFF", "GRID_UNDEF"]
