"""The allocation-free scan, fl_prefix_sum_noalloc, called through the C ABI.

It exists for host applications that cannot let this library allocate
device memory (an engine or plugin host that owns the whole device budget,
or a real-time loop where cudaMalloc/cudaFree would synchronise the device).
Its scratch is a fixed array inside the library, so it must give exactly
the offsets of the system scan, fl_prefix_sum_cells, on caller-owned
buffers -- here on two calls in a row, since every call reuses (and must
first clear) that array. Kept in its own file, collected last.
"""
from __future__ import annotations

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import _lib, scenes

from helpers import assert_bit_equal

pytestmark = pytest.mark.gpu


def _scan(d_counts, d_offsets, n, zero_offsets, d_status):
    return _lib.lib().fl_prefix_sum_noalloc(d_counts.data_ptr(), d_offsets.data_ptr(), n, zero_offsets,
                                            d_status.data_ptr(), None)


def test_noalloc_scan_matches_the_system_scan_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    # reference result: the system scan of a real grid (352,800 cells, 87 tiles)
    sc = scenes.wave_tank(n=300_000)
    with F.FluidSystem(sc.params, sc.n) as s:
        s.SetParticles(sc.pos, sc.vel, sc.veval, clr=sc.clr)
        _, _, cnt = s.InsertParticlesCUDA(readback=True)
        want_excl = s.PrefixSumCellsCUDA(1, readback=True)
        want_incl = s.PrefixSumCellsCUDA(0, readback=True)
        s.Sync()
    n = cnt.size
    d_cnt = torch.from_numpy(cnt.view(np.int32).copy()).cuda()
    d_status = torch.zeros(1, dtype=torch.int32, device="cuda")
    for call in range(2):
        for zero_offsets, want in ((1, want_excl), (0, want_incl)):
            d_off = torch.full((n,), -1, dtype=torch.int32, device="cuda")
            assert _scan(d_cnt, d_off, n, zero_offsets, d_status) == 0, _lib.lib().fl_last_error()
            torch.cuda.synchronize()
            assert_bit_equal(d_off.cpu().numpy().view(np.uint32), want,
                             f"call {call}, zero_offsets={zero_offsets}")
    assert int(d_status.item()) == 0


def test_noalloc_scan_ragged_and_limit():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    for n in (1, 4095, 4097, 12_345):
        cnt = rng.integers(0, 60, size=n, dtype=np.uint32)
        d_cnt = torch.from_numpy(cnt.view(np.int32)).cuda()
        d_off = torch.empty(n, dtype=torch.int32, device="cuda")
        d_status = torch.zeros(1, dtype=torch.int32, device="cuda")
        assert _scan(d_cnt, d_off, n, 1, d_status) == 0
        torch.cuda.synchronize()
        want = (np.cumsum(cnt, dtype=np.uint64) - cnt).astype(np.uint32)
        assert_bit_equal(d_off.cpu().numpy().view(np.uint32), want, f"n={n}")
    # beyond the fixed scratch: rejected before any GPU work
    big = F.lib().fl_prefix_sum_noalloc(None, None, 4194305, 1, None, None)
    assert big == -1 and b"exceed" in F.lib().fl_last_error()


def test_noalloc_scan_wait_runs_out_and_is_reported():
    """The scan's bounded look-back wait, made to run out on purpose: the
    test hook withholds tile 0 (one CTA fewer, every index in bounds) with a
    256-poll limit. The call returns, FL_DEV_SPIN_TIMEOUT lands in d_status,
    and the next ordinary call (which clears the shared scratch) scans
    correctly again."""
    torch = pytest.importorskip("torch")
    n = 3 * 4096 + 5
    cnt = np.random.default_rng(8).integers(0, 40, size=n, dtype=np.uint32)
    d_cnt = torch.from_numpy(cnt.view(np.int32)).cuda()
    d_off = torch.empty(n, dtype=torch.int32, device="cuda")
    d_status = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = _lib.lib()
    assert lib.fl_test_scan_noalloc_timeout(d_cnt.data_ptr(), d_off.data_ptr(), n, d_status.data_ptr(), 256,
                                            None) == 0, lib.fl_last_error()
    torch.cuda.synchronize()
    assert int(d_status.item()) & 0x1
    d_status.zero_()
    assert _scan(d_cnt, d_off, n, 1, d_status) == 0
    torch.cuda.synchronize()
    want = (np.cumsum(cnt, dtype=np.uint64) - cnt).astype(np.uint32)
    assert_bit_equal(d_off.cpu().numpy().view(np.uint32), want, "scan after the timed-out one")
    assert int(d_status.item()) == 0
