"""ctypes view of the C ABI declared in include/fluid_gb300.h.

The structs here mirror the header field by field; `tests/test_capi_cpu.py`
checks their sizes against the compiled library's own `sizeof` report so that a
drift between the two fails loudly.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfluidgb.so")

FGB_OK = 0
FGB_ERR_INVALID = 1
FGB_ERR_CUDA = 2
FGB_ERR_OOM = 3
FGB_ERR_CAPACITY = 4
FGB_ERR_TIMEOUT = 5
FGB_ERR_UNSUPPORTED = 6
FGB_ERR_BUDGET = 7

PROFILE_REF = 0
PROFILE_BASELINE = 1
TYPE_FLUID = 0
TYPE_OBSTACLE = 1
MAX_WELLS = 16

PROBE_KEYS = 1
PROBE_ORDER = 2
PROBE_CELLS = 3
PROBE_LAMBDA = 4
PROBE_DENSITY = 5
PROBE_LATTICE = 6
PROBE_CUBE_CASES = 7
PROBE_LIST_COUNT = 8
PROBE_LIST_VALID = 9
PROBE_DISPLACEMENT = 10
PROBE_NEAR_ROW = 11

f3 = ctypes.c_float * 3


class Params(ctypes.Structure):
    _fields_ = [
        ("h", ctypes.c_float),
        ("profile", ctypes.c_int32),
        ("rho0", ctypes.c_float),
        ("cfm_epsilon", ctypes.c_float),
        ("corr_k", ctypes.c_float),
        ("corr_n", ctypes.c_float),
        ("corr_delta_q", ctypes.c_float),
        ("xsph_c", ctypes.c_float),
        ("vorticity_epsilon", ctypes.c_float),
        ("velocity_damping", ctypes.c_float),
        ("mc_particle_size", ctypes.c_float),
        ("mc_particle_influence", ctypes.c_float),
    ]


class Well(ctypes.Structure):
    _fields_ = [("centre", f3), ("force", ctypes.c_float)]


class Config(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_float),
        ("scale", ctypes.c_float),
        ("resolution", ctypes.c_float),
        ("isolevel", ctypes.c_float),
        ("iterations", ctypes.c_uint32),
        ("surface", ctypes.c_uint32),
        ("constant_force", f3),
        ("min_bound", f3),
        ("max_bound", f3),
        ("sphere_enabled", ctypes.c_int32),
        ("sphere", ctypes.c_float * 4),
        ("n_wells", ctypes.c_uint32),
        ("wells", Well * MAX_WELLS),
    ]


class Particles(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_size_t),
        ("id", ctypes.POINTER(ctypes.c_uint64)),
        ("type", ctypes.POINTER(ctypes.c_int32)),
        ("mass", ctypes.POINTER(ctypes.c_float)),
        ("position", ctypes.POINTER(ctypes.c_float)),
        ("velocity", ctypes.POINTER(ctypes.c_float)),
        ("colour", ctypes.POINTER(ctypes.c_uint32)),
    ]


class Triangle(ctypes.Structure):
    _fields_ = [("a", f3), ("b", f3), ("c", f3)]


class MeshTriangle(ctypes.Structure):
    _fields_ = [("v", ctypes.c_float * 9), ("n", ctypes.c_float * 9), ("c", ctypes.c_uint32 * 3)]


class Mesh(ctypes.Structure):
    _fields_ = [
        ("triangles", ctypes.POINTER(MeshTriangle)),
        ("n", ctypes.c_size_t),
        ("capacity", ctypes.c_size_t),
    ]


class GridInfo(ctypes.Structure):
    _fields_ = [
        ("min_extent", f3),
        ("extent", ctypes.c_uint32 * 3),
        ("table_offset", ctypes.c_uint64),
        ("table_size", ctypes.c_uint64),
        ("morton_bits", ctypes.c_uint32),
        ("scene_bits", ctypes.c_uint32),
        ("lattice", ctypes.c_uint32 * 3),
        ("lattice_origin", f3),
        ("lattice_step", ctypes.c_float),
    ]


SERVE_WAITING = 0
SERVE_ACTIVE = 1
SERVE_DONE = 2


class ServeOptions(ctypes.Structure):
    _fields_ = [
        ("budget_bytes", ctypes.c_uint64),
        ("max_active", ctypes.c_uint32),
        ("one_at_a_time", ctypes.c_uint32),
        ("tick_particles", ctypes.c_uint64),
        ("max_steps_per_tick", ctypes.c_uint32),
    ]


class ServeResult(ctypes.Structure):
    _fields_ = [
        ("ticket", ctypes.c_uint64),
        ("n", ctypes.c_uint64),
        ("steps", ctypes.c_uint32),
        ("status", ctypes.c_int32),
        ("triangles", ctypes.c_uint64),
        ("t_submit", ctypes.c_double),
        ("t_admit", ctypes.c_double),
        ("t_done", ctypes.c_double),
    ]


class ServeStats(ctypes.Structure):
    _fields_ = [
        ("ticks", ctypes.c_uint64),
        ("particle_steps", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("rejected", ctypes.c_uint64),
        ("failed", ctypes.c_uint64),
        ("active", ctypes.c_uint64),
        ("waiting", ctypes.c_uint64),
        ("used_bytes", ctypes.c_uint64),
        ("budget_bytes", ctypes.c_uint64),
        ("rebuilds", ctypes.c_uint64),
        ("busy_seconds", ctypes.c_double),
        ("rebuild_seconds", ctypes.c_double),
        ("elapsed_seconds", ctypes.c_double),
    ]


class Source(ctypes.Structure):
    _fields_ = [("centre", f3), ("velocity", f3), ("rate", ctypes.c_uint64), ("tag", ctypes.c_uint64),
                ("colour", ctypes.c_uint32)]


class Drain(ctypes.Structure):
    _fields_ = [("centre", f3), ("width", ctypes.c_float), ("depth", ctypes.c_float)]


class Query(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("point", ctypes.c_float * 3)]


class QueryResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("point", ctypes.c_float * 3), ("neighbours", ctypes.c_uint64),
                ("average_colour", ctypes.c_uint32)]


class Records(ctypes.Structure):
    _fields_ = [("base", ctypes.c_void_p), ("n", ctypes.c_size_t), ("stride", ctypes.c_uint32),
                ("id_bytes", ctypes.c_uint32), ("id", ctypes.c_int32), ("type", ctypes.c_int32),
                ("mass", ctypes.c_int32), ("position", ctypes.c_int32), ("velocity", ctypes.c_int32),
                ("colour", ctypes.c_int32)]


# numpy record type with the layout of fluid::Particle<size_t, float> (fluid.hpp:52-62)
# built against GLM's packed vectors: id, type, mass, position, velocity, colour
PARTICLE_RECORD = np.dtype({"names": ["id", "type", "mass", "position", "velocity", "colour"],
                            "formats": [np.uint64, np.int32, np.float32, (np.float32, 3), (np.float32, 3), np.uint32],
                            "offsets": [0, 8, 12, 16, 28, 40], "itemsize": 48})


def records_view(rec):
    """Records struct over a numpy array of PARTICLE_RECORD (kept alive by the caller)."""
    r = Records()
    r.base = rec.ctypes.data
    r.n = len(rec)
    r.stride = rec.dtype.itemsize
    r.id_bytes = 8
    f = rec.dtype.fields
    r.id, r.type, r.mass = f["id"][1], f["type"][1], f["mass"][1]
    r.position, r.velocity, r.colour = f["position"][1], f["velocity"][1], f["colour"][1]
    return r


def to_records(parts):
    n = len(parts["mass"])
    rec = np.zeros(n, PARTICLE_RECORD)
    rec["id"], rec["type"], rec["mass"], rec["colour"] = parts["id"], parts["type"], parts["mass"], parts["colour"]
    rec["position"] = parts["position"].reshape(n, 3)
    rec["velocity"] = parts["velocity"].reshape(n, 3)
    return rec


def from_records(rec):
    return {"id": rec["id"].copy(), "type": rec["type"].copy(), "mass": rec["mass"].copy(),
            "position": np.ascontiguousarray(rec["position"]).ravel().copy(),
            "velocity": np.ascontiguousarray(rec["velocity"]).ravel().copy(), "colour": rec["colour"].copy()}


class TuneResult(ctypes.Structure):
    _fields_ = [("block", ctypes.c_uint32), ("skin", ctypes.c_float), ("ms_per_step", ctypes.c_float),
                ("trials", ctypes.c_uint32), ("steps", ctypes.c_uint32), ("persistent", ctypes.c_uint32),
                ("particles_per_thread", ctypes.c_uint32), ("verlet", ctypes.c_uint32)]


P = ctypes.POINTER
c_void_p = ctypes.c_void_p

_SIGS = {
    "fgb_version": (ctypes.c_int, []),
    "fgb_last_error": (ctypes.c_char_p, []),
    "fgb_struct_sizes": (ctypes.c_int, [P(ctypes.c_uint64), ctypes.c_int]),
    "fgb_params_default": (None, [P(Params), ctypes.c_int32, ctypes.c_float]),
    "fgb_config_default": (None, [P(Config), ctypes.c_int32]),
    "fgb_create": (ctypes.c_int, [P(Params), P(c_void_p)]),
    "fgb_destroy": (ctypes.c_int, [c_void_p]),
    "fgb_set_stream": (ctypes.c_int, [c_void_p, c_void_p]),
    "fgb_advance": (ctypes.c_int, [c_void_p, P(Config), P(Particles), P(Triangle), ctypes.c_size_t, P(Mesh)]),
    "fgb_mesh_free": (None, [P(Mesh)]),
    "fgb_batch_create": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(ctypes.c_uint64), P(Config), P(c_void_p)]),
    "fgb_batch_destroy": (ctypes.c_int, [c_void_p]),
    "fgb_batch_upload": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(Particles)]),
    "fgb_batch_set_colliders": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(Triangle), ctypes.c_size_t]),
    "fgb_batch_step": (ctypes.c_int, [c_void_p, ctypes.c_uint32]),
    "fgb_batch_download": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(Particles)]),
    "fgb_batch_surface": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(Mesh)]),
    "fgb_batch_surface_all": (ctypes.c_int, [c_void_p, P(ctypes.c_uint64)]),
    "fgb_batch_surface_fetch": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(Mesh)]),
    "fgb_batch_sync": (ctypes.c_int, [c_void_p]),
    "fgb_batch_error_flags": (ctypes.c_int, [c_void_p, P(ctypes.c_uint32)]),
    "fgb_batch_row_stats": (ctypes.c_int, [c_void_p, P(ctypes.c_uint32), ctypes.c_uint32]),
    "fgb_batch_host_io": (ctypes.c_int, [c_void_p, P(ctypes.c_int)]),
    "fgb_batch_prepare": (ctypes.c_int, [c_void_p]),
    "fgb_batch_launch_count": (ctypes.c_uint64, [c_void_p]),
    "fgb_batch_set_timing": (ctypes.c_int, [c_void_p, ctypes.c_int]),
    "fgb_batch_autotune": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(TuneResult)]),
    "fgb_batch_sources_drains": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(Source), ctypes.c_uint32, P(Drain),
                                                ctypes.c_uint32, P(ctypes.c_uint64)]),
    "fgb_batch_stage_times": (ctypes.c_int, [c_void_p, P(ctypes.c_float), ctypes.c_uint32, P(ctypes.c_uint32)]),
    "fgb_batch_probe_size": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(ctypes.c_uint64)]),
    "fgb_batch_probe": (ctypes.c_int, [c_void_p, ctypes.c_uint32, c_void_p, ctypes.c_uint64]),
    "fgb_batch_grid_info": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(GridInfo)]),
    "fgb_batch_copy_scene": (ctypes.c_int, [c_void_p, ctypes.c_uint32, c_void_p, ctypes.c_uint32]),
    "fgb_scene_footprint": (ctypes.c_int, [c_void_p, P(Config), ctypes.c_uint64, ctypes.c_int, P(ctypes.c_uint64)]),
    "fgb_serve_create": (ctypes.c_int, [c_void_p, P(ServeOptions), P(c_void_p)]),
    "fgb_serve_submit": (ctypes.c_int, [c_void_p, P(Config), P(Particles), ctypes.c_uint32, ctypes.c_int,
                                        P(ctypes.c_uint64)]),
    "fgb_serve_poll": (ctypes.c_int, [c_void_p, ctypes.c_uint64, P(ServeResult)]),
    "fgb_serve_fetch": (ctypes.c_int, [c_void_p, ctypes.c_uint64, P(Particles), P(Mesh)]),
    "fgb_serve_get_stats": (ctypes.c_int, [c_void_p, P(ServeStats)]),
    "fgb_serve_step_latencies": (ctypes.c_int, [c_void_p, P(ctypes.c_double), ctypes.c_uint64,
                                                P(ctypes.c_uint64)]),
    "fgb_serve_tick_particles": (ctypes.c_int, [c_void_p, P(ctypes.c_uint64), ctypes.c_uint64,
                                                P(ctypes.c_uint64)]),
    "fgb_serve_tick_starts": (ctypes.c_int, [c_void_p, P(ctypes.c_double), ctypes.c_uint64,
                                             P(ctypes.c_uint64)]),
    "fgb_serve_tick_scenes": (ctypes.c_int, [c_void_p, P(ctypes.c_uint32), ctypes.c_uint64,
                                             P(ctypes.c_uint64)]),
    "fgb_serve_tick_steps": (ctypes.c_int, [c_void_p, P(ctypes.c_uint32), ctypes.c_uint64,
                                            P(ctypes.c_uint64)]),
    "fgb_serve_drain": (ctypes.c_int, [c_void_p, ctypes.c_double]),
    "fgb_serve_destroy": (ctypes.c_int, [c_void_p]),
    "fgb_exclusive_scan_u32_noalloc": (ctypes.c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_uint64, c_void_p]),
    "fgb_wire_particles": (ctypes.c_int, [P(Particles), ctypes.c_int64, c_void_p, ctypes.c_uint64,
                                          P(ctypes.c_uint64)]),
    "fgb_wire_triangles": (ctypes.c_int, [P(Mesh), ctypes.c_int64, c_void_p, ctypes.c_uint64, P(ctypes.c_uint64)]),
    "fgb_batch_wire_particles": (ctypes.c_int, [c_void_p, ctypes.c_uint32, ctypes.c_int64, c_void_p,
                                                ctypes.c_uint64, P(ctypes.c_uint64)]),
    "fgb_batch_wire_surface": (ctypes.c_int, [c_void_p, ctypes.c_uint32, ctypes.c_int64, c_void_p,
                                              ctypes.c_uint64, P(ctypes.c_uint64)]),
    "fgb_weld_mesh": (ctypes.c_int, [P(Mesh), c_void_p, c_void_p, P(ctypes.c_uint64)]),
    "fgb_batch_weld_surface": (ctypes.c_int, [c_void_p, ctypes.c_uint32, c_void_p, c_void_p, P(ctypes.c_uint64)]),
    "fgb_radix_sort_scratch_bytes": (ctypes.c_uint64, [ctypes.c_uint64]),
    "fgb_radix_sort_pairs_u32": (ctypes.c_int, [c_void_p, c_void_p, c_void_p, c_void_p, ctypes.c_uint64,
                                                ctypes.c_uint32, c_void_p, ctypes.c_uint64, c_void_p]),
    "fgb_scan_scratch_bytes": (ctypes.c_uint64, [ctypes.c_uint64]),
    "fgb_exclusive_scan_u32": (ctypes.c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_uint64, c_void_p,
                                              ctypes.c_uint64, c_void_p]),
    "fgb_radix_sort_error": (ctypes.c_int, [c_void_p, ctypes.c_uint64, c_void_p, P(ctypes.c_uint32)]),
    "fgb_scan_error": (ctypes.c_int, [c_void_p, ctypes.c_uint64, c_void_p, P(ctypes.c_uint32)]),
    "fgb_scan_noalloc_error": (ctypes.c_int, [c_void_p, P(ctypes.c_uint32)]),
    "fgb_test_lookback_fault": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32]),
    "fgb_host_ready_pages": (ctypes.c_int, [c_void_p, ctypes.c_size_t, ctypes.c_int, P(ctypes.c_uint64)]),
    "fgb_advance_records": (ctypes.c_int, [c_void_p, P(Config), P(Records), P(Triangle), ctypes.c_size_t, P(Query),
                                           ctypes.c_size_t, P(QueryResult), P(ctypes.c_size_t), P(Mesh)]),
    "fgb_batch_query": (ctypes.c_int, [c_void_p, ctypes.c_uint32, P(Query), ctypes.c_size_t, P(QueryResult),
                                       P(ctypes.c_size_t)]),
}

_lib = None


class FluidError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libfluidgb error {code}: {msg}")
        self.code = code


def load(path=None):
    """Load the CUDA library; raises if it is missing (there is no CPU fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(p)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc):
    if rc != FGB_OK:
        msg = load().fgb_last_error()
        raise FluidError(rc, msg.decode() if msg else "")
    return rc


def exported_symbols():
    """Names of every function declared in include/fluid_gb300.h."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "fluid_gb300.h")
    src = open(hdr).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fgb_[a-z0-9_]+)\s*\(", src)))


def params(profile=PROFILE_BASELINE, h=0.1):
    p = Params()
    load().fgb_params_default(ctypes.byref(p), profile, h)
    return p


def particles_view(arrs):
    """Particles struct pointing at numpy arrays (kept alive by the caller)."""
    pv = Particles()
    pv.n = len(arrs["mass"])
    pv.id = arrs["id"].ctypes.data_as(P(ctypes.c_uint64))
    pv.type = arrs["type"].ctypes.data_as(P(ctypes.c_int32))
    pv.mass = arrs["mass"].ctypes.data_as(P(ctypes.c_float))
    pv.position = arrs["position"].ctypes.data_as(P(ctypes.c_float))
    pv.velocity = arrs["velocity"].ctypes.data_as(P(ctypes.c_float))
    pv.colour = arrs["colour"].ctypes.data_as(P(ctypes.c_uint32))
    return pv


def mesh_to_numpy(mesh):
    n = int(mesh.n)
    if n == 0:
        return np.zeros((0, 21), np.float32)
    buf = ctypes.cast(mesh.triangles, P(ctypes.c_float * (21 * n))).contents
    return np.frombuffer(buf, dtype=np.float32).reshape(n, 21).copy()


def default_params(profile=PROFILE_BASELINE, h=0.1):
    """Pure-Python copy of fgb_params_default (a CPU test keeps the two equal)."""
    p = Params()
    p.h = h
    p.profile = profile
    p.corr_n = 4.0
    p.mc_particle_size = 25.0       # oclsph.hpp:672
    p.mc_particle_influence = 0.5   # oclsph.hpp:673
    p.vorticity_epsilon = 0.0005    # oclsph_kernel.h:29
    if profile == PROFILE_REF:      # oclsph_kernel.h:20-31
        p.rho0 = 6378.0
        p.cfm_epsilon = 600.0
        p.corr_k = 0.0001
        p.corr_delta_q = 0.3
        p.xsph_c = 0.00001
        p.velocity_damping = 0.49
    else:
        p.rho0 = 1000.0
        p.cfm_epsilon = 100.0
        p.corr_k = 0.1
        p.corr_delta_q = 0.2
        p.xsph_c = 0.01
        p.velocity_damping = 1.0
    return p
