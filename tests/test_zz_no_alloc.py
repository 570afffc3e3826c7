"""The allocation-free scan entry point, for callers that cannot call cudaMalloc
(a host whose memory manager owns every device allocation, a plugin host that
forbids its plugins to allocate, or a real-time loop where an allocation could
block or fail).

Called through the C ABI and compared with fgb_exclusive_scan_u32 (caller scratch)
on two calls in a row: the second call must not see stale look-back state left in
the shared static scratch by the first.  Collected last so that a failure here
comes after every other test has run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from libfluid_gb300 import capi

pytestmark = pytest.mark.gpu


def _scan_reference(torch, lib, x):
    n = x.numel()
    out = torch.empty_like(x)
    tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    sb = lib.fgb_scan_scratch_bytes(n)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    capi.check(lib.fgb_exclusive_scan_u32(x.data_ptr(), out.data_ptr(), tot.data_ptr(), n, scratch.data_ptr(), sb,
                                          torch.cuda.current_stream().cuda_stream))
    return out, tot


def test_noalloc_scan_matches_scan_with_scratch_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = capi.load()
    fn = lib.fgb_exclusive_scan_u32_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(123)
    # two calls in a row of different sizes: the larger first, so that the second
    # would read leftover tile status if the shared scratch were not cleared
    for n in (5_000_000, 1_234_567):
        x = torch.from_numpy(rng.integers(0, 9, n).astype(np.int32)).cuda()
        out = torch.empty_like(x)
        tot = torch.zeros(1, dtype=torch.int32, device="cuda")
        capi.check(fn(x.data_ptr(), out.data_ptr(), tot.data_ptr(), n, stream))
        ref_out, ref_tot = _scan_reference(torch, lib, x)
        torch.cuda.synchronize()
        assert torch.equal(out, ref_out)
        assert int(tot.item()) == int(ref_tot.item()) == int(x.sum().item())


def test_noalloc_scan_rejects_sizes_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = capi.load()
    fn = lib.fgb_exclusive_scan_u32_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    x = torch.zeros(16, dtype=torch.int32, device="cuda")
    # the size check comes before any device access, so a short buffer is safe here
    rc = fn(x.data_ptr(), x.data_ptr(), None, 16777216 + 1, torch.cuda.current_stream().cuda_stream)
    assert rc == capi.FGB_ERR_CAPACITY
    assert b"FGB_SCAN_NOALLOC_MAX_N" in lib.fgb_last_error()
