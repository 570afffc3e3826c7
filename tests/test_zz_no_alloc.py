"""The allocation-free scan entry point, for callers that cannot call cudaMalloc
(a host whose memory manager owns every device allocation, a plugin host that
forbids its plugins to allocate, or a real-time loop where an allocation could
block or fail).

Called through the C ABI and compared with a numpy cumsum and with
fgb_exclusive_scan_u32 (caller scratch) on calls in a row: a later call must not
see stale look-back state left in the shared static scratch by an earlier one.
The sizes cover the empty scan, exact multiples of the 4096-item tile and the
documented maximum, where the last tile's status word sits at the end of the fixed
array.  Collected last so that a failure here comes after every other test has
run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from libfluid_gb300 import capi

pytestmark = pytest.mark.gpu

MAX_N = 16777216


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = capi.load()
    return torch, lib, torch.cuda.current_stream().cuda_stream


def _cumsum(x):
    if len(x) == 0:
        return np.zeros(0, np.uint32), 0
    c = np.cumsum(x.astype(np.uint64))
    return np.concatenate([[0], c[:-1]]).astype(np.uint32), int(c[-1]) & 0xFFFFFFFF


def _scan_with_scratch(torch, lib, stream, x):
    n = x.numel()
    out = torch.empty_like(x)
    tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    sb = lib.fgb_scan_scratch_bytes(n)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    capi.check(lib.fgb_exclusive_scan_u32(x.data_ptr(), out.data_ptr(), tot.data_ptr(), n, scratch.data_ptr(), sb,
                                          stream))
    return out, tot


def _noalloc_flags(lib, stream):
    f = ctypes.c_uint32(0xDEAD)
    capi.check(lib.fgb_scan_noalloc_error(stream, ctypes.byref(f)))
    return f.value


def test_noalloc_scan_matches_cumsum_and_scan_with_scratch_on_calls_in_a_row(env):
    torch, lib, stream = env
    rng = np.random.default_rng(123)
    # the larger first, so that a later call would read leftover tile status if the
    # shared scratch were not cleared; 4096 * k sizes end exactly on a tile
    for n in (5_000_000, 1_234_567, 4096 * 7, 4096, 1, 0, 4096 * 300 + 1):
        x_np = rng.integers(0, 9, n).astype(np.uint32)
        x = torch.from_numpy(x_np.view(np.int32)).cuda()
        out = torch.empty_like(x)
        tot = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        capi.check(lib.fgb_exclusive_scan_u32_noalloc(x.data_ptr(), out.data_ptr(), tot.data_ptr(), n, stream))
        ref_out, ref_tot = _scan_with_scratch(torch, lib, stream, x)
        torch.cuda.synchronize()
        want, total = _cumsum(x_np)
        got = out.cpu().numpy().view(np.uint32)
        assert (got == want).all(), n
        assert torch.equal(out, ref_out), n
        assert int(tot.cpu().numpy().view(np.uint32)[0]) == int(ref_tot.cpu().numpy().view(np.uint32)[0]) == total
        assert _noalloc_flags(lib, stream) == 0


def test_noalloc_scan_at_its_maximum_size_and_without_a_total(env):
    torch, lib, stream = env
    rng = np.random.default_rng(7)
    x_np = rng.integers(0, 2, MAX_N).astype(np.uint32)  # the total stays below 2^32
    x = torch.from_numpy(x_np.view(np.int32)).cuda()
    for with_total in (True, False):
        out = torch.empty_like(x)
        tot = torch.zeros(1, dtype=torch.int32, device="cuda")
        capi.check(lib.fgb_exclusive_scan_u32_noalloc(x.data_ptr(), out.data_ptr(),
                                                      tot.data_ptr() if with_total else None, MAX_N, stream))
        torch.cuda.synchronize()
        want, total = _cumsum(x_np)
        assert (out.cpu().numpy().view(np.uint32) == want).all()
        assert int(tot.item()) == (total if with_total else 0)
        assert _noalloc_flags(lib, stream) == 0


def test_noalloc_scan_rejects_sizes_beyond_its_maximum(env):
    torch, lib, stream = env
    x = torch.zeros(16, dtype=torch.int32, device="cuda")
    # the size check comes before any device access, so a short buffer is safe here
    rc = lib.fgb_exclusive_scan_u32_noalloc(x.data_ptr(), x.data_ptr(), None, MAX_N + 1, stream)
    assert rc == capi.FGB_ERR_CAPACITY
    assert b"FGB_SCAN_NOALLOC_MAX_N" in lib.fgb_last_error()


def test_noalloc_scan_reports_a_lookback_that_ran_out(env):
    # one tile never publishes and the spin limit is small (fgb_test_lookback_fault):
    # the next tile's wait runs out, the call returns, and the error query sees it
    torch, lib, stream = env
    x_np = np.ones(4 * 4096, np.uint32)
    x = torch.from_numpy(x_np.view(np.int32)).cuda()
    out = torch.empty_like(x)
    capi.check(lib.fgb_test_lookback_fault(0, 4096))
    try:
        capi.check(lib.fgb_exclusive_scan_u32_noalloc(x.data_ptr(), out.data_ptr(), None, len(x_np), stream))
    finally:
        capi.check(lib.fgb_test_lookback_fault(0xFFFFFFFF, 0))
    assert _noalloc_flags(lib, stream) & (1 << 1)
    assert _noalloc_flags(lib, stream) == 0  # read and cleared
    capi.check(lib.fgb_exclusive_scan_u32_noalloc(x.data_ptr(), out.data_ptr(), None, len(x_np), stream))
    torch.cuda.synchronize()
    assert (out.cpu().numpy().view(np.uint32) == np.arange(len(x_np), dtype=np.uint32)).all()
    assert _noalloc_flags(lib, stream) == 0
