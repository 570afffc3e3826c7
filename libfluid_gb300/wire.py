"""Packed record streams (fgb_wire_* / fgb_batch_wire_* in include/fluid_gb300.h).

The byte layout of the reference demo's memory-mapped result files
(samples/structures.hpp particleDef / meshTriangleDef / queryResultDef / headerDef,
written by mmf::writer::writePacked): a 24-byte header, then the records, each
field in declaration order with no padding, little-endian.  The numpy dtypes below
read such a stream (or a file the reference wrote); the functions write one.
"""
import ctypes
import time

import numpy as np

from . import capi

HEADER = np.dtype([("timestamp", "<i8"), ("entries", "<u8"), ("written", "<u8")])
PARTICLE = np.dtype([("id", "<u8"), ("type", "<i4"), ("mass", "<f4"), ("colour", "<u4"),
                     ("position", "<f4", (3,)), ("velocity", "<f4", (3,))])
TRIANGLE = np.dtype([("v", "<f4", (3, 3)), ("n", "<f4", (3, 3)), ("c", "<u4", (3,))])
QUERY = np.dtype([("id", "<u8"), ("point", "<f4", (3,)), ("neighbours", "<u8"), ("average_colour", "<u4")])


def now_ms():
    return int(time.time() * 1000)


def read(buf, record):
    """(header, records) of a stream in `buf` (bytes, bytearray, memoryview, mmap)."""
    h = np.frombuffer(buf, HEADER, count=1)[0]
    recs = np.frombuffer(buf, record, count=int(h["entries"]), offset=HEADER.itemsize)
    return h, recs


def _run(fn, *args):
    size = ctypes.c_uint64()
    capi.check(fn(*args, None, 0, ctypes.byref(size)))
    out = bytearray(size.value)
    dst = (ctypes.c_char * len(out)).from_buffer(out)
    capi.check(fn(*args, dst, len(out), ctypes.byref(size)))
    return out


def particles(parts, timestamp_ms=None, lib=None):
    """Stream of host particle arrays (the dict form of libfluid_gb300.scenes)."""
    lib = lib or capi.load()
    pv = capi.particles_view(parts)
    ts = now_ms() if timestamp_ms is None else timestamp_ms
    return _run(lib.fgb_wire_particles, ctypes.byref(pv), ts)


def triangles(tris, timestamp_ms=None, lib=None):
    """Stream of an (n, 21) float32 triangle array as returned by Batch.surface."""
    lib = lib or capi.load()
    tris = np.ascontiguousarray(tris, np.float32)
    m = capi.Mesh()
    m.n = len(tris)
    m.capacity = len(tris)
    m.triangles = ctypes.cast(tris.ctypes.data, ctypes.POINTER(capi.MeshTriangle)) if len(tris) else None
    ts = now_ms() if timestamp_ms is None else timestamp_ms
    return _run(lib.fgb_wire_triangles, ctypes.byref(m), ts)


def batch_particles(batch, k, timestamp_ms=None):
    """Stream of resident scene k, packed on the device."""
    ts = now_ms() if timestamp_ms is None else timestamp_ms
    return _run(batch.lib.fgb_batch_wire_particles, batch.handle, k, ts)


def batch_surface(batch, k, timestamp_ms=None):
    """Triangles of scene k from the batch's last surface_all()."""
    ts = now_ms() if timestamp_ms is None else timestamp_ms
    return _run(batch.lib.fgb_batch_wire_surface, batch.handle, k, ts)


def queries(results, timestamp_ms=None):
    """Stream of query results [(id, (x, y, z), neighbours, average_colour), ...]
    (answered on the host by the C++ adapter; packed here in numpy)."""
    recs = np.zeros(len(results), QUERY)
    for i, (qid, point, nb, colour) in enumerate(results):
        recs[i] = (qid, point, nb, colour)
    ts = now_ms() if timestamp_ms is None else timestamp_ms
    head = np.array([(ts, len(recs), len(recs))], HEADER)
    return bytearray(head.tobytes() + recs.tobytes())
