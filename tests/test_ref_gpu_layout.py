"""The reference's GPU module is driven through a field-by-field restatement
of its FParams and FBufs blocks (oracle/ref_gpu.py). Every offset is checked
here against the reference header itself, through the host build of the
reference kernels, and the launch shapes against computeNumBlocks."""
from __future__ import annotations

import ctypes as C

import pytest

from oracle import oracle as O
from oracle import ref_gpu as R


def test_fparams_and_fbufs_layout_match_the_reference_header():
    if not O.ref_available():
        pytest.skip("host build of the reference kernels absent (reference tree not present at build time)")
    lib = O.ref()
    lib.ref_layout.restype = C.c_long
    lib.ref_layout.argtypes = [C.c_char_p]
    for name, _ in R.RefFParams._fields_:
        assert lib.ref_layout(name.encode()) == getattr(R.RefFParams, name).offset, name
    assert lib.ref_layout(b"sizeof FParams") == C.sizeof(R.RefFParams)
    assert lib.ref_layout(b"sizeof FBufs") == C.sizeof(R.RefFBufs)
    assert lib.ref_layout(b"FBufs.mgpu") == R.RefFBufs.mgpu.offset


def test_launch_shapes_follow_compute_num_blocks():
    """computeNumBlocks (fluids4.0/fluid_system.cpp:2193-2197) with the 512
    threads per block of FluidSetupCUDA."""
    assert R.num_blocks(4_000_000, 512) == (512, 7813)
    assert R.num_blocks(32_768, 512) == (512, 64)
    assert R.num_blocks(100, 512) == (100, 1)
    assert R.num_blocks(0, 512) == (0, 1)


def test_parameter_block_from_derived_params():
    from fluids3_gb300 import scenes
    sc = scenes.dam_break()
    p = sc.params
    f = R.fparams_from(p, sc.n)
    assert f.pnum == sc.n and f.gridTotal == p.gridTotal and f.gridAdjCnt == p.gridAdjCnt == 8
    assert list(f.gridAdj[:8]) == list(p.gridAdj[:8])
    assert f.rd2 == p.rd2 and f.vterm == p.vterm and list(f.gridDelta) == list(p.gridDelta)
    assert (f.numThreads, f.numBlocks) == (512, 64) and f.szPnts == 32_768
