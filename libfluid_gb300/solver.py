"""Python mirror of libfluid's solver interface over the C ABI.

`SphSolver.advance(config, particles, colliders)` has the meaning of
fluid::SphSolver<size_t,float>::advance (include/fluid/fluid.hpp:222-232): the
particles are advanced one step and written back reordered into Morton order,
and when the config asks for a surface the marching-cubes triangles are
returned.  Errors raise `capi.FluidError` carrying the library's status code,
as the reference throws.  There is no CPU fallback: a missing CUDA library or
device raises.
"""
import atexit
import ctypes
import weakref

import numpy as np

from . import capi

_P = ctypes.POINTER
_live_solvers = weakref.WeakSet()


@atexit.register
def _close_all():
    # release device objects before the CUDA runtime shuts down at process exit
    for s in list(_live_solvers):
        s.close()


def _tri_array(colliders):
    if colliders is None or len(colliders) == 0:
        return None, 0
    arr = np.ascontiguousarray(colliders, dtype=np.float32).reshape(-1, 9)
    return arr, len(arr)


class SphSolver:
    """Replaces ocl::SphSolver(h, kernelPath, device) (include/fluid/oclsph.hpp:170-189)."""

    def __init__(self, h=0.1, profile=capi.PROFILE_BASELINE, params=None):
        self.lib = capi.load()
        self.params = params if params is not None else capi.params(profile, h)
        self._h = ctypes.c_void_p()
        self._batches = weakref.WeakSet()
        self._servers = weakref.WeakSet()
        capi.check(self.lib.fgb_create(ctypes.byref(self.params), ctypes.byref(self._h)))
        _live_solvers.add(self)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr):
        capi.check(self.lib.fgb_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def advance(self, config, particles, colliders=None):
        """One frame on a dict of numpy arrays (updated in place, Morton order);
        returns the mesh as an (n, 21) float32 array (v0 v1 v2 n0 n1 n2 + colours as
        raw uint32 bits) when config.surface is set, else None."""
        pv = capi.particles_view(particles)
        tris, ntris = _tri_array(colliders)
        mesh = capi.Mesh()
        tp = tris.ctypes.data_as(_P(capi.Triangle)) if tris is not None else None
        rc = self.lib.fgb_advance(self._h, ctypes.byref(config), ctypes.byref(pv), tp, ntris,
                                  ctypes.byref(mesh))
        try:
            capi.check(rc)
            return capi.mesh_to_numpy(mesh) if config.surface else None
        finally:
            self.lib.fgb_mesh_free(ctypes.byref(mesh))

    def advance_records(self, config, records, colliders=None, queries=None):
        """One frame on a numpy array of capi.PARTICLE_RECORD (read and written in
        place, Morton order) with cell queries [(id, (x, y, z))]: returns (mesh or
        None, [(id, point, neighbours, average_colour)])."""
        rv = capi.records_view(records)
        tris, ntris = _tri_array(colliders)
        tp = tris.ctypes.data_as(_P(capi.Triangle)) if tris is not None else None
        queries = list(queries or [])
        nq = len(queries)
        qs = (capi.Query * max(nq, 1))()
        for i, (qid, pt) in enumerate(queries):
            qs[i].id = qid
            qs[i].point[:] = pt
        res = (capi.QueryResult * max(nq, 1))()
        nres = ctypes.c_size_t()
        mesh = capi.Mesh()
        rc = self.lib.fgb_advance_records(self._h, ctypes.byref(config), ctypes.byref(rv), tp, ntris, qs, nq, res,
                                          ctypes.byref(nres), ctypes.byref(mesh))
        try:
            capi.check(rc)
            out = [(int(res[i].id), tuple(res[i].point), int(res[i].neighbours), int(res[i].average_colour))
                   for i in range(nres.value)]
            return (capi.mesh_to_numpy(mesh) if config.surface else None), out
        finally:
            self.lib.fgb_mesh_free(ctypes.byref(mesh))

    def close(self):
        if self._h:
            # the library destroys the solver's batches with it
            for sv in list(self._servers):  # a server's worker uses the solver
                sv.close()
            for b in list(self._batches):
                b._h = ctypes.c_void_p()
            self.lib.fgb_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Resident scenes advanced together (one launch per stage for all scenes)."""

    def __init__(self, solver, scenes):
        self.solver = solver
        self.lib = solver.lib
        self.n_scenes = len(scenes)
        counts = (ctypes.c_uint64 * self.n_scenes)(*[len(p["mass"]) for p, _ in scenes])
        cfgs = (capi.Config * self.n_scenes)(*[c for _, c in scenes])
        self.counts = [int(c) for c in counts]
        self.configs = [c for _, c in scenes]
        self._h = ctypes.c_void_p()
        capi.check(self.lib.fgb_batch_create(solver.handle, self.n_scenes, counts, cfgs, ctypes.byref(self._h)))
        solver._batches.add(self)
        for k, (parts, _) in enumerate(scenes):
            self.upload(k, parts)

    def upload(self, k, parts):
        pv = capi.particles_view(parts)
        capi.check(self.lib.fgb_batch_upload(self._h, k, ctypes.byref(pv)))

    def set_colliders(self, k, colliders):
        tris, ntris = _tri_array(colliders)
        tp = tris.ctypes.data_as(_P(capi.Triangle)) if tris is not None else None
        capi.check(self.lib.fgb_batch_set_colliders(self._h, k, tp, ntris))

    @property
    def handle(self):
        return self._h

    def step(self, steps=1):
        capi.check(self.lib.fgb_batch_step(self._h, steps))

    def sync(self):
        capi.check(self.lib.fgb_batch_sync(self._h))

    def sources_drains(self, k, sources=(), drains=()):
        """Apply sources [(centre, velocity, rate, tag, colour)] and drains
        [(centre, width)] to resident scene k on the device; returns its new count."""
        srcs = (capi.Source * max(len(sources), 1))()
        for i, (centre, vel, rate, tag, colour) in enumerate(sources):
            srcs[i].centre[:] = centre
            srcs[i].velocity[:] = vel
            srcs[i].rate, srcs[i].tag, srcs[i].colour = rate, tag, colour
        drs = (capi.Drain * max(len(drains), 1))()
        for i, (centre, width) in enumerate(drains):
            drs[i].centre[:] = centre
            drs[i].width = width
        count = ctypes.c_uint64()
        capi.check(self.lib.fgb_batch_sources_drains(self._h, k, srcs, len(sources), drs, len(drains),
                                                     ctypes.byref(count)))
        self.counts[k] = int(count.value)
        return self.counts[k]

    def autotune(self, steps_per_trial=3):
        """Pick the fastest launch shape on this batch's next steps (they are ordinary
        steps) and cache it in the solver for its size bucket; returns TuneResult."""
        r = capi.TuneResult()
        capi.check(self.lib.fgb_batch_autotune(self._h, steps_per_trial, ctypes.byref(r)))
        return r

    def download(self, k):
        n = self.counts[k]
        out = {
            "id": np.zeros(n, np.uint64),
            "type": np.zeros(n, np.int32),
            "mass": np.zeros(n, np.float32),
            "position": np.zeros(3 * n, np.float32),
            "velocity": np.zeros(3 * n, np.float32),
            "colour": np.zeros(n, np.uint32),
        }
        pv = capi.particles_view(out)
        capi.check(self.lib.fgb_batch_download(self._h, k, ctypes.byref(pv)))
        return out

    def surface(self, k):
        mesh = capi.Mesh()
        try:
            capi.check(self.lib.fgb_batch_surface(self._h, k, ctypes.byref(mesh)))
            return capi.mesh_to_numpy(mesh)
        finally:
            self.lib.fgb_mesh_free(ctypes.byref(mesh))

    def surface_all(self):
        counts = (ctypes.c_uint64 * self.n_scenes)()
        capi.check(self.lib.fgb_batch_surface_all(self._h, counts))
        return [int(c) for c in counts]

    def surface_fetch(self, k):
        mesh = capi.Mesh()
        try:
            capi.check(self.lib.fgb_batch_surface_fetch(self._h, k, ctypes.byref(mesh)))
            return capi.mesh_to_numpy(mesh)
        finally:
            self.lib.fgb_mesh_free(ctypes.byref(mesh))

    def probe(self, what, dtype):
        nbytes = ctypes.c_uint64()
        capi.check(self.lib.fgb_batch_probe_size(self._h, what, ctypes.byref(nbytes)))
        out = np.zeros(int(nbytes.value) // np.dtype(dtype).itemsize, dtype)
        capi.check(self.lib.fgb_batch_probe(self._h, what, out.ctypes.data_as(ctypes.c_void_p), nbytes.value))
        return out

    def grid_info(self, k):
        gi = capi.GridInfo()
        capi.check(self.lib.fgb_batch_grid_info(self._h, k, ctypes.byref(gi)))
        return gi

    def host_io_direct(self):
        """True where uploads and downloads are kernels on the caller's arrays."""
        d = ctypes.c_int()
        capi.check(self.lib.fgb_batch_host_io(self._h, ctypes.byref(d)))
        return bool(d.value)

    def query(self, k, queries):
        """Cell queries [(id, (x, y, z))] of scene k against the grid of the last step."""
        nq = len(queries)
        qs = (capi.Query * max(nq, 1))()
        for i, (qid, pt) in enumerate(queries):
            qs[i].id = qid
            qs[i].point[:] = pt
        res = (capi.QueryResult * max(nq, 1))()
        nres = ctypes.c_size_t()
        capi.check(self.lib.fgb_batch_query(self._h, k, qs, nq, res, ctypes.byref(nres)))
        return [(int(res[i].id), tuple(res[i].point), int(res[i].neighbours), int(res[i].average_colour))
                for i in range(nres.value)]

    def error_flags(self):
        f = ctypes.c_uint32()
        capi.check(self.lib.fgb_batch_error_flags(self._h, ctypes.byref(f)))
        return int(f.value)

    def row_stats(self):
        """(warps of checked passes on near rows, warps that filtered, filtering
        particles on their Verlet list, walking particles) since the last call; zeros
        unless FGB_ROW_STATS=1 was set when the batch was created."""
        out = (ctypes.c_uint32 * 4)()
        capi.check(self.lib.fgb_batch_row_stats(self._h, out, 4))
        return tuple(int(x) for x in out)

    def set_timing(self, on=True):
        capi.check(self.lib.fgb_batch_set_timing(self._h, 1 if on else 0))

    def stage_times(self):
        """Per-stage milliseconds of the last step: predict, sort, reorder,
        (lambda, delta) per iteration, then vorticity and vorticity apply."""
        buf = (ctypes.c_float * 64)()
        cnt = ctypes.c_uint32()
        capi.check(self.lib.fgb_batch_stage_times(self._h, buf, 64, ctypes.byref(cnt)))
        return [float(buf[i]) for i in range(cnt.value)]

    @property
    def launches(self):
        return int(self.lib.fgb_batch_launch_count(self._h))

    def close(self):
        # a closed solver has already destroyed its batches
        if self._h and self.solver._h:
            self.lib.fgb_batch_destroy(self._h)
        self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
