"""Vertex welding (fgb_weld_mesh / fgb_batch_weld_surface in include/fluid_gb300.h).

An index buffer for a triangle soup with the meaning of geometry::indexVBO2
(include/fluid/geometry.hpp:152-166): vertices in triangle order, a position
byte-identical to an earlier one reusing its index, distinct positions in order of
first appearance.  Computed on the GPU.
"""
import ctypes

import numpy as np

from . import capi


def _out(n_tris):
    return np.zeros(3 * n_tris, np.uint32), np.zeros(9 * n_tris, np.float32)


def weld(tris, lib=None):
    """(indices (3 n,) uint32, vertices (m, 3) float32) of an (n, 21) float32 mesh."""
    lib = lib or capi.load()
    tris = np.ascontiguousarray(tris, np.float32)
    n = len(tris)
    idx, verts = _out(n)
    m = capi.Mesh()
    m.n = m.capacity = n
    m.triangles = ctypes.cast(tris.ctypes.data, ctypes.POINTER(capi.MeshTriangle)) if n else None
    count = ctypes.c_uint64()
    capi.check(lib.fgb_weld_mesh(ctypes.byref(m), idx.ctypes.data_as(ctypes.c_void_p),
                                 verts.ctypes.data_as(ctypes.c_void_p), ctypes.byref(count)))
    return idx, verts[:3 * count.value].reshape(-1, 3)


def batch_weld(batch, k, n_tris):
    """Weld scene k's triangles of the batch's last surface_all() (n_tris of them)
    where they lie on the device."""
    idx, verts = _out(n_tris)
    count = ctypes.c_uint64()
    capi.check(batch.lib.fgb_batch_weld_surface(batch.handle, k, idx.ctypes.data_as(ctypes.c_void_p),
                                                verts.ctypes.data_as(ctypes.c_void_p), ctypes.byref(count)))
    return idx, verts[:3 * count.value].reshape(-1, 3)
