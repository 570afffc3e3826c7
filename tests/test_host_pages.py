"""Host-side page readying (fgb_host_ready_pages), the step fgb_advance takes on the
caller's arrays before its kernels read and write them in place over the coherent
link.  A page that is not resident can still hold the caller's data (swapped-out
memory, a file mapping whose page was evicted), so for arrays that are also inputs
the touch must keep every byte.  CPU only: no kernel runs."""
import ctypes
import mmap
import os
import tempfile

import numpy as np
import pytest

from libfluid_gb300 import capi

PAGE = mmap.PAGESIZE


@pytest.fixture(scope="module")
def lib():
    from libfluid_gb300 import build
    build.build()
    return capi.load()


def _resident(buf_addr, nbytes):
    libc = ctypes.CDLL(None, use_errno=True)
    libc.mincore.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_char_p]
    pages = (nbytes + PAGE - 1) // PAGE
    vec = ctypes.create_string_buffer(pages)
    if libc.mincore(ctypes.c_void_p(buf_addr), nbytes, vec) != 0:
        return None
    return np.frombuffer(vec.raw, np.uint8) & 1


def _address(mm):
    view = np.frombuffer(mm, np.uint8)
    addr = view.ctypes.data
    del view
    return addr


def _evicted_file_mapping(data):
    """A shared mapping of a file holding `data` whose pages were dropped from the
    page cache, or None where the file system keeps them (tmpfs)."""
    for d in (tempfile.gettempdir(), os.path.dirname(os.path.abspath(__file__))):
        fd, path = tempfile.mkstemp(dir=d)
        try:
            os.write(fd, data.tobytes())
            os.fsync(fd)
            mm = mmap.mmap(fd, data.nbytes, mmap.MAP_SHARED, mmap.PROT_READ | mmap.PROT_WRITE)
            addr = _address(mm)
            mm.madvise(mmap.MADV_DONTNEED)
            os.posix_fadvise(fd, 0, 0, os.POSIX_FADV_DONTNEED)
            res = _resident(addr, data.nbytes)
            if res is not None and (res == 0).sum() >= len(res) // 2:
                return fd, path, mm, addr
            mm.close()
        except (OSError, AttributeError, ValueError):
            pass
        os.close(fd)
        os.unlink(path)
    return None


def test_keep_contents_preserves_evicted_file_pages(lib):
    rng = np.random.default_rng(5)
    data = rng.integers(1, 256, 64 * PAGE, dtype=np.uint8)  # no zero byte anywhere
    got = _evicted_file_mapping(data)
    if got is None:
        pytest.skip("no file system here lets its pages be evicted")
    fd, path, mm, addr = got
    try:
        before = _resident(addr, data.nbytes)
        touched = ctypes.c_uint64(0)
        capi.check(lib.fgb_host_ready_pages(ctypes.c_void_p(addr), data.nbytes, 1, ctypes.byref(touched)))
        assert touched.value == int((before == 0).sum()) > 0
        assert (_resident(addr, data.nbytes) == 1).all()
        assert mm[:] == data.tobytes(), "an input page lost its contents"
        mm.flush()
        os.posix_fadvise(fd, 0, 0, os.POSIX_FADV_DONTNEED)
        assert np.array_equal(np.fromfile(path, np.uint8), data), "the file changed"
    finally:
        mm.close()
        os.close(fd)
        os.unlink(path)


def test_output_pages_of_fresh_memory_are_touched_once(lib):
    n = 32 * PAGE
    mm = mmap.mmap(-1, n)
    try:
        addr = _address(mm)
        touched = ctypes.c_uint64(0)
        capi.check(lib.fgb_host_ready_pages(ctypes.c_void_p(addr), n, 0, ctypes.byref(touched)))
        assert touched.value == 32
        assert (_resident(addr, n) == 1).all()
        assert not any(mm[:])
        capi.check(lib.fgb_host_ready_pages(ctypes.c_void_p(addr), n, 0, ctypes.byref(touched)))
        assert touched.value == 0  # resident now: nothing to do
    finally:
        mm.close()


def test_null_range_is_rejected(lib):
    assert lib.fgb_host_ready_pages(None, 16, 1, None) == capi.FGB_ERR_INVALID
    capi.check(lib.fgb_host_ready_pages(None, 0, 1, None))
