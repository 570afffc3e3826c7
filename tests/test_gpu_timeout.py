"""Bounded device waits that run out.  The radix sort and the scans wait on earlier
tiles in their decoupled look-back; every such wait is bounded, and when it gives
up the kernel raises an error flag and returns instead of hanging.  Here the wait is
made to run out on purpose with fgb_test_lookback_fault: one tile never publishes
its status (a flag that nothing sets) and the spin limit is small, so the tile after
it gives up within milliseconds.  Each test checks that the error comes back as a
status, that the call returned, and that the next normal call works.  Nothing here
faults, traps or hangs the GPU: the kernels' own bounds keep every store in range.
"""
import ctypes

import numpy as np
import pytest

from libfluid_gb300 import capi, scenes
from libfluid_gb300.solver import Batch, SphSolver

pytestmark = pytest.mark.gpu

SORT_FLAG = 1 << 0
SCAN_FLAG = 1 << 1
SPINS = 4096


@pytest.fixture()
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    yield torch
    capi.check(capi.load().fgb_test_lookback_fault(0xFFFFFFFF, 0))


def _fault(on):
    lib = capi.load()
    capi.check(lib.fgb_test_lookback_fault(0 if on else 0xFFFFFFFF, SPINS if on else 0))


def _sort(torch, keys, key_bits):
    lib = capi.load()
    n = len(keys)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.arange(n, dtype=torch.int32, device="cuda")
    ok, ov = torch.empty_like(dk), torch.empty_like(dv)
    sb = lib.fgb_radix_sort_scratch_bytes(n)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    capi.check(lib.fgb_radix_sort_pairs_u32(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n, key_bits,
                                            scratch.data_ptr(), sb, stream))
    flags = ctypes.c_uint32(0xDEAD)
    capi.check(lib.fgb_radix_sort_error(scratch.data_ptr(), n, stream, ctypes.byref(flags)))
    return ok.cpu().numpy().view(np.uint32), ov.cpu().numpy().view(np.uint32), flags.value


def _scan(torch, x):
    lib = capi.load()
    n = len(x)
    dx = torch.from_numpy(x.view(np.int32)).cuda()
    out = torch.empty_like(dx)
    tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    sb = lib.fgb_scan_scratch_bytes(n)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    capi.check(lib.fgb_exclusive_scan_u32(dx.data_ptr(), out.data_ptr(), tot.data_ptr(), n, scratch.data_ptr(), sb,
                                          stream))
    flags = ctypes.c_uint32(0xDEAD)
    capi.check(lib.fgb_scan_error(scratch.data_ptr(), n, stream, ctypes.byref(flags)))
    return out.cpu().numpy().view(np.uint32), flags.value


def test_sort_lookback_that_runs_out_is_reported_and_the_next_sort_is_right(torch_cuda):
    rng = np.random.default_rng(3)
    n = 5 * 4096 + 17  # six tiles: tile 0 is skipped, tile 1 waits on it
    keys = rng.integers(0, 1 << 24, n, dtype=np.uint64).astype(np.uint32)
    _fault(True)
    k, v, flags = _sort(torch_cuda, keys, 24)
    assert flags & SORT_FLAG, f"no timeout flag ({flags:#x})"
    _fault(False)
    k, v, flags = _sort(torch_cuda, keys, 24)
    assert flags == 0
    order = np.argsort(keys, kind="stable")
    assert (k == keys[order]).all() and (v == order).all()


def test_scan_lookback_that_runs_out_is_reported_and_the_next_scan_is_right(torch_cuda):
    rng = np.random.default_rng(4)
    x = rng.integers(0, 9, 3 * 4096 + 5).astype(np.uint32)
    _fault(True)
    out, flags = _scan(torch_cuda, x)
    assert flags & SCAN_FLAG, f"no timeout flag ({flags:#x})"
    _fault(False)
    out, flags = _scan(torch_cuda, x)
    assert flags == 0
    want = np.concatenate([[0], np.cumsum(x.astype(np.uint64))[:-1]]).astype(np.uint32)
    assert (out == want).all()


def _scene():
    return scenes.dam_break((24, 24, 24), (2.4, 2.4, 2.4), seed=91)  # 13 824 particles: 4 sort tiles


def test_batch_step_and_sync_report_a_timed_out_sort_then_a_new_batch_steps_normally(torch_cuda):
    params = capi.params(capi.PROFILE_BASELINE, 0.1)
    parts, cfg = _scene()
    solver = SphSolver(params=params)
    _fault(True)  # captured into this batch's step graphs
    bad = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    bad.step(1)  # queued: no step has finished yet
    with pytest.raises(capi.FluidError) as e:
        bad.sync()
    assert e.value.code == capi.FGB_ERR_TIMEOUT
    # the flag stays until read: no further step is queued on suspect state
    with pytest.raises(capi.FluidError) as e:
        bad.step(1)
    assert e.value.code == capi.FGB_ERR_TIMEOUT
    assert bad.error_flags() & SORT_FLAG
    bad.close()
    _fault(False)
    good = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    good.step(2)
    good.sync()
    assert good.error_flags() == 0
    ref_solver = SphSolver(params=params)
    ref = Batch(ref_solver, [(scenes.copy_particles(parts), cfg)])
    ref.step(2)
    a, b = good.download(0), ref.download(0)
    for f in ("id", "position", "velocity"):
        assert (a[f] == b[f]).all(), f
    for x in (good, ref):
        x.close()
    solver.close()
    ref_solver.close()


def test_advance_raises_on_a_timed_out_frame_and_the_next_solver_is_fine(torch_cuda):
    params = capi.params(capi.PROFILE_BASELINE, 0.1)
    parts, cfg = _scene()
    _fault(True)
    solver = SphSolver(params=params)
    with pytest.raises(capi.FluidError) as e:
        solver.advance(cfg, scenes.copy_particles(parts))
    assert e.value.code == capi.FGB_ERR_TIMEOUT
    solver.close()
    _fault(False)
    solver = SphSolver(params=params)
    got = scenes.copy_particles(parts)
    solver.advance(cfg, got)
    solver.advance(cfg, got)
    ref_solver = SphSolver(params=params)
    want = scenes.copy_particles(parts)
    ref_solver.advance(cfg, want)
    ref_solver.advance(cfg, want)
    for f in ("id", "position", "velocity"):
        assert (got[f] == want[f]).all(), f
    solver.close()
    ref_solver.close()
