"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, as the checker or the timed CPU baseline; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_shim.so")

_lib = None
_ref = None


def build(quiet=True):
    """Compile the oracle (and the reference shim where the reference tree exists)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        from libfluid_gb300 import capi
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        vp = ctypes.c_void_p
        L.orc_morton.restype = ctypes.c_uint32
        L.orc_morton.argtypes = [ctypes.c_uint32] * 3
        L.orc_morton_decode.restype = ctypes.c_uint32
        L.orc_morton_decode.argtypes = [ctypes.c_uint32, ctypes.c_int]
        L.orc_mc_tables.argtypes = [vp, vp, vp]
        L.orc_poly6.restype = ctypes.c_float
        L.orc_poly6.argtypes = [P(capi.Params), ctypes.c_float]
        L.orc_spiky_scale.restype = ctypes.c_float
        L.orc_spiky_scale.argtypes = [P(capi.Params), ctypes.c_float]
        L.orc_grid_geometry.argtypes = [P(capi.Params), P(capi.Config), vp]
        L.orc_key.restype = ctypes.c_uint32
        L.orc_key.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.orc_lattice_geometry.argtypes = [P(capi.Params), P(capi.Config), vp, vp]
        L.orc_step.restype = ctypes.c_int
        L.orc_step.argtypes = [P(capi.Params), P(capi.Config), ctypes.c_size_t, vp, vp, vp, vp, vp, vp,
                               vp, ctypes.c_size_t, vp]
        L.orc_surface.restype = ctypes.c_size_t
        L.orc_surface.argtypes = [P(capi.Params), P(capi.Config), ctypes.c_size_t, vp, vp, vp, vp, vp,
                                  vp, vp, vp, ctypes.c_size_t]
        L.orc_march.restype = ctypes.c_size_t
        L.orc_march.argtypes = [P(capi.Params), P(capi.Config), vp, vp, vp, vp, vp, ctypes.c_size_t]
        L.orc_weld.restype = ctypes.c_size_t
        L.orc_weld.argtypes = [vp, ctypes.c_size_t, vp, vp]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


REF_KERNELS_LIB = os.path.join(HERE, "_ref", "libref_kernels.so")
_refk = None


def ref_kernels():
    """The reference's own OpenCL kernel bodies compiled as C++ (ref_kernels.cpp),
    or None when not built (no reference tree)."""
    global _refk
    if _refk is None and os.path.exists(REF_KERNELS_LIB):
        K = ctypes.CDLL(REF_KERNELS_LIB)
        vp = ctypes.c_void_p
        K.refk_h.restype = ctypes.c_float
        K.refk_solve.restype = ctypes.c_int
        K.refk_solve.argtypes = [ctypes.c_uint32, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_uint32, vp,
                                 ctypes.c_uint32, vp, vp, vp, vp, vp, vp]
        K.refk_lattice.restype = ctypes.c_int
        K.refk_lattice.argtypes = [ctypes.c_uint32, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_float, vp, vp]
        K.refk_cube_counts.restype = ctypes.c_int
        K.refk_cube_counts.argtypes = [vp, ctypes.c_float, vp, vp]
        K.refk_mc_eval.restype = ctypes.c_size_t
        K.refk_mc_eval.argtypes = [vp, vp, vp, ctypes.c_float, vp, vp, vp, ctypes.c_size_t]
        _refk = K
    return _refk


def ref_solve(K, cfg, keys, type_, mass, colour, pstar, position, velocity, ext, colliders=None):
    """Run the reference's sph_diffuse, lambda/delta iterations and sph_finalise on a
    predicted, sorted state; returns dict(pstar, position, velocity, lambda, colour)."""
    n = len(keys)
    c = lambda a, t: np.ascontiguousarray(a, t)  # noqa: E731
    keys, type_, mass, colour = c(keys, np.uint32), c(type_, np.int32), c(mass, np.float32), c(colour, np.uint32)
    pstar, position, velocity = c(pstar, np.float32), c(position, np.float32), c(velocity, np.float32)
    tris = c(colliders if colliders is not None else np.zeros((0, 9)), np.float32).reshape(-1, 9)
    cf = np.array([cfg.dt, cfg.scale, *cfg.min_bound, *cfg.max_bound], np.float32)
    ex = np.array(list(ext), np.uint32)
    out = {k: np.zeros(3 * n, np.float32) for k in ("pstar", "position", "velocity")}
    out["lambda"] = np.zeros(n, np.float32)
    out["colour"] = np.zeros(n, np.uint32)
    rc = K.refk_solve(n, _ptr(keys), _ptr(type_), _ptr(mass), _ptr(colour), _ptr(pstar), _ptr(position),
                      _ptr(velocity), _ptr(tris) if len(tris) else None, len(tris), _ptr(cf), cfg.iterations,
                      _ptr(ex), _ptr(out["pstar"]), _ptr(out["position"]), _ptr(out["velocity"]),
                      _ptr(out["lambda"]), _ptr(out["colour"]))
    if rc != 0:
        raise RuntimeError("reference kernels: a particle's neighbour cells leave the grid table")
    return out


def ref_surface(K, params, cfg, parts):
    """The reference's mc_lattice, mc_size and mc_eval on the current state, sampled
    with a grid built over these positions; returns (lattice[samples, 4] in the
    oracle's sample order, colours, cube triangle counts, triangles[n, 21])."""
    g = grid(params, cfg)
    l = lattice(params, cfg)
    n = len(parts["mass"])
    pos = np.asarray(parts["position"], np.float32).reshape(-1, 3)
    keys = np.array([lib().orc_key(ctypes.byref(g), params.h, *(pos[i] / cfg.scale)) for i in range(n)],
                    np.uint32)
    order = np.argsort(keys, kind="stable")
    sizes = np.array(list(l.size), np.uint32)
    samples = int(sizes.prod())
    lat = np.zeros(4 * samples, np.float32)
    lcol = np.zeros(samples, np.uint32)
    mc = np.array([cfg.resolution, params.mc_particle_size, params.mc_particle_influence, cfg.isolevel], np.float32)
    ext = np.array(list(g.ext), np.uint32)
    mn = np.array(list(g.min_ext), np.float32)
    c = np.ascontiguousarray
    K.refk_lattice(n, _ptr(c(keys[order])), _ptr(c(parts["type"][order], np.int32)),
                   _ptr(c(pos[order].reshape(-1), np.float32)), _ptr(c(parts["colour"][order], np.uint32)),
                   _ptr(ext), _ptr(mn), _ptr(sizes), _ptr(mc), cfg.scale, _ptr(lat), _ptr(lcol))
    cubes = int(np.prod(sizes - 1))
    counts = np.zeros(max(cubes, 1), np.uint32)
    K.refk_cube_counts(_ptr(sizes), cfg.isolevel, _ptr(lat), _ptr(counts))
    cap = int(counts[:cubes].sum())
    tris = np.zeros((max(cap, 1), 21), np.float32)
    total = K.refk_mc_eval(_ptr(sizes), _ptr(mn), _ptr(mc), cfg.scale, _ptr(lat), _ptr(lcol), _ptr(tris), cap)
    return lat.reshape(-1, 4), lcol, counts[:cubes], tris[:total]


REF_CPU_LIB = os.path.join(HERE, "_ref", "libref_cpusph.so")


class RefCpuSolver:
    """The reference's own OpenMP solver, cpu::SphSolver (include/fluid/cpusph.hpp),
    built by oracle/Makefile from the patched copy in oracle/_ref/src: the
    benchmark's timed reference arm.  It keeps the reference's constants and has no
    wells, colliders, colours or surface."""

    def __init__(self, h, parts):
        K = ctypes.CDLL(REF_CPU_LIB)
        vp = ctypes.c_void_p
        K.refcpu_create.restype = vp
        K.refcpu_create.argtypes = [ctypes.c_float]
        K.refcpu_destroy.argtypes = [vp]
        K.refcpu_threads.restype = ctypes.c_int
        K.refcpu_threads.argtypes = [ctypes.c_int]
        K.refcpu_load.argtypes = [vp, ctypes.c_size_t, vp, vp, vp, vp, vp, vp]
        K.refcpu_advance.restype = ctypes.c_double
        K.refcpu_advance.argtypes = [vp, vp, ctypes.c_int]
        K.refcpu_store.argtypes = [vp, vp, vp]
        self.K = K
        self.n = len(parts["mass"])
        self.h = K.refcpu_create(h)
        c = np.ascontiguousarray
        K.refcpu_load(self.h, self.n, _ptr(c(parts["id"], np.uint64)), _ptr(c(parts["type"], np.int32)),
                      _ptr(c(parts["mass"], np.float32)), _ptr(c(parts["position"], np.float32)),
                      _ptr(c(parts["velocity"], np.float32)), _ptr(c(parts["colour"], np.uint32)))

    @staticmethod
    def available():
        return os.path.exists(REF_CPU_LIB)

    def threads(self, n=0):
        return int(self.K.refcpu_threads(n))

    def advance(self, cfg, steps=1):
        """`steps` calls of advance(); returns their wall time in seconds."""
        c = np.array([cfg.dt, cfg.scale, cfg.iterations, *cfg.constant_force, *cfg.min_bound, *cfg.max_bound],
                     np.float32)
        return float(self.K.refcpu_advance(self.h, _ptr(c), steps))

    def state(self):
        pos = np.zeros(3 * self.n, np.float32)
        vel = np.zeros(3 * self.n, np.float32)
        self.K.refcpu_store(self.h, _ptr(pos), _ptr(vel))
        return pos, vel

    def close(self):
        if self.h:
            self.K.refcpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def ref_lib():
    """The reference's own curves.h / mctable.hpp / mc.h, or None when not built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        R = ctypes.CDLL(REF_LIB)
        R.ref_morton.restype = ctypes.c_uint64
        R.ref_morton.argtypes = [ctypes.c_uint64] * 3
        R.ref_morton_decode.restype = ctypes.c_uint64
        R.ref_morton_decode.argtypes = [ctypes.c_uint64, ctypes.c_int]
        for f in ("ref_edge_table", "ref_num_verts", "ref_cl_edge_table", "ref_cl_num_verts"):
            getattr(R, f).restype = ctypes.c_int
            getattr(R, f).argtypes = [ctypes.c_int]
        for f in ("ref_tri_table", "ref_cl_tri_table"):
            getattr(R, f).restype = ctypes.c_int
            getattr(R, f).argtypes = [ctypes.c_int, ctypes.c_int]
        _ref = R
    return _ref


class Grid(ctypes.Structure):
    _fields_ = [("min_ext", ctypes.c_float * 3), ("ext", ctypes.c_uint32 * 3), ("table_n", ctypes.c_uint32)]


class Lattice(ctypes.Structure):
    _fields_ = [("size", ctypes.c_uint32 * 3), ("origin", ctypes.c_float * 3), ("step", ctypes.c_float)]


class Probe(ctypes.Structure):
    _fields_ = [("keys", ctypes.c_void_p), ("order", ctypes.c_void_p), ("cells", ctypes.c_void_p),
                ("lambda_", ctypes.c_void_p), ("density", ctypes.c_void_p), ("pstar", ctypes.c_void_p),
                ("omega", ctypes.c_void_p)]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def mc_tables():
    em = np.zeros(256, np.uint16)
    nv = np.zeros(256, np.uint8)
    tri = np.zeros((256, 16), np.uint8)
    lib().orc_mc_tables(_ptr(em), _ptr(nv), _ptr(tri))
    return em, nv, tri


def grid(params, cfg):
    g = Grid()
    lib().orc_grid_geometry(ctypes.byref(params), ctypes.byref(cfg), ctypes.byref(g))
    return g


def lattice(params, cfg):
    g = grid(params, cfg)
    l = Lattice()
    lib().orc_lattice_geometry(ctypes.byref(params), ctypes.byref(cfg), ctypes.byref(g), ctypes.byref(l))
    return l


def step(params, cfg, parts, colliders=None, probe=False):
    """One step in place on a dict of arrays (see libfluid_gb300.scenes.block).
    Returns the probe dict when probe=True."""
    n = len(parts["mass"])
    pr = None
    out = None
    if probe:
        g = grid(params, cfg)
        out = {
            "keys": np.zeros(n, np.uint32),
            "order": np.zeros(n, np.uint32),
            "cells": np.zeros(2 * g.table_n, np.uint32),
            "lambda": np.zeros(n, np.float32),
            "density": np.zeros(n, np.float32),
            "pstar": np.zeros(3 * n, np.float32),
            "omega": np.zeros(4 * n, np.float32),
        }
        pr = Probe(_ptr(out["keys"]), _ptr(out["order"]), _ptr(out["cells"]), _ptr(out["lambda"]),
                   _ptr(out["density"]), _ptr(out["pstar"]), _ptr(out["omega"]))
    tris = None
    ntris = 0
    if colliders is not None and len(colliders):
        tris = np.ascontiguousarray(colliders, np.float32)
        ntris = len(tris)
    rc = lib().orc_step(ctypes.byref(params), ctypes.byref(cfg), n, _ptr(parts["id"]), _ptr(parts["type"]),
                        _ptr(parts["mass"]), _ptr(parts["position"]), _ptr(parts["velocity"]),
                        _ptr(parts["colour"]), _ptr(tris) if tris is not None else None, ntris,
                        ctypes.byref(pr) if pr is not None else None)
    if rc != 0:
        raise RuntimeError("oracle step failed")
    return out


def surface(params, cfg, parts, want_lattice=False):
    """Marching cubes of the current state: (triangles[n,21], lattice, colours, cases)."""
    n = len(parts["mass"])
    l = lattice(params, cfg)
    samples = l.size[0] * l.size[1] * l.size[2]
    cubes = max(l.size[0] - 1, 0) * max(l.size[1] - 1, 0) * max(l.size[2] - 1, 0)
    lat = np.zeros(4 * samples, np.float32)
    lcol = np.zeros(samples, np.uint32)
    cases = np.zeros(max(cubes, 1), np.uint8)
    L = lib()
    total = L.orc_surface(ctypes.byref(params), ctypes.byref(cfg), n, _ptr(parts["type"]), _ptr(parts["mass"]),
                          _ptr(parts["position"]), _ptr(parts["colour"]), _ptr(lat), _ptr(lcol),
                          _ptr(cases), None, 0)
    tris = np.zeros((max(total, 1), 21), np.float32)
    total2 = L.orc_march(ctypes.byref(params), ctypes.byref(cfg), ctypes.byref(l), _ptr(lat), _ptr(lcol),
                         None, _ptr(tris), total)
    assert total2 == total
    tris = tris[:total]
    if want_lattice:
        return tris, lat.reshape(-1, 4), lcol, cases[:cubes]
    return tris


def march(params, cfg, lat, lcol):
    """Marching cubes of a given lattice (stage-wise parity)."""
    l = lattice(params, cfg)
    cubes = (l.size[0] - 1) * (l.size[1] - 1) * (l.size[2] - 1)
    cases = np.zeros(max(cubes, 1), np.uint8)
    lat = np.ascontiguousarray(lat, np.float32)
    lcol = np.ascontiguousarray(lcol, np.uint32)
    L = lib()
    total = L.orc_march(ctypes.byref(params), ctypes.byref(cfg), ctypes.byref(l), _ptr(lat), _ptr(lcol),
                        _ptr(cases), None, 0)
    tris = np.zeros((max(total, 1), 21), np.float32)
    L.orc_march(ctypes.byref(params), ctypes.byref(cfg), ctypes.byref(l), _ptr(lat), _ptr(lcol), None,
                _ptr(tris), total)
    return tris[:total], cases[:cubes]


def weld(tris):
    """(indices, vertices) of an (n, 21) float32 triangle array (geometry.hpp:152-166)."""
    tris = np.ascontiguousarray(tris, np.float32)
    n = len(tris)
    idx = np.zeros(3 * n, np.uint32)
    verts = np.zeros(9 * n, np.float32)
    m = lib().orc_weld(_ptr(tris), n, _ptr(idx), _ptr(verts)) if n else 0
    return idx, verts[:3 * m].reshape(-1, 3)


def set_threads(n):
    lib().orc_set_threads(int(n))


def num_threads():
    return int(lib().orc_num_threads())
