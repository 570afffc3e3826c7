"""Python view of the serving loop (fgb_serve_* in include/fluid_gb300.h)."""
import ctypes

import numpy as np

from . import capi


class Server:
    """Continuous-batching request loop over one solver.

    submit() copies a scene and returns a ticket; the library's worker thread admits
    scenes against the HBM budget, packs resident scenes into groups of at most
    tick_particles particles, advances one group per tick (round robin) by one
    batched step, or by up to max_steps_per_tick steps when the group holds less than
    half of tick_particles, and, when a scene has run its steps, extracts its surface
    (on request) and keeps its final state for fetch()."""

    def __init__(self, solver, budget_bytes=150 << 30, max_active=256, one_at_a_time=False, tick_particles=0,
                 max_steps_per_tick=0):
        self.solver = solver
        self.lib = solver.lib
        opt = capi.ServeOptions(budget_bytes, max_active, 1 if one_at_a_time else 0, tick_particles,
                                max_steps_per_tick)
        self._h = ctypes.c_void_p()
        capi.check(self.lib.fgb_serve_create(solver.handle, ctypes.byref(opt), ctypes.byref(self._h)))
        solver._servers.add(self)
        self._n = {}

    def submit(self, cfg, parts, steps, want_mesh=False):
        pv = capi.particles_view(parts)
        t = ctypes.c_uint64()
        capi.check(self.lib.fgb_serve_submit(self._h, ctypes.byref(cfg), ctypes.byref(pv), steps,
                                             1 if want_mesh else 0, ctypes.byref(t)))
        self._n[t.value] = len(parts["mass"])
        return int(t.value)

    def poll(self, ticket):
        r = capi.ServeResult()
        capi.check(self.lib.fgb_serve_poll(self._h, ticket, ctypes.byref(r)))
        return r

    def fetch(self, ticket):
        """(particles dict, mesh array) of a finished request; releases it."""
        n = self._n.pop(ticket)
        out = {"id": np.zeros(n, np.uint64), "type": np.zeros(n, np.int32), "mass": np.zeros(n, np.float32),
               "position": np.zeros(3 * n, np.float32), "velocity": np.zeros(3 * n, np.float32),
               "colour": np.zeros(n, np.uint32)}
        pv = capi.particles_view(out)
        mesh = capi.Mesh()
        try:
            capi.check(self.lib.fgb_serve_fetch(self._h, ticket, ctypes.byref(pv), ctypes.byref(mesh)))
            return out, capi.mesh_to_numpy(mesh)
        finally:
            self.lib.fgb_mesh_free(ctypes.byref(mesh))

    def drain(self, timeout=600.0):
        capi.check(self.lib.fgb_serve_drain(self._h, timeout))

    def stats(self):
        s = capi.ServeStats()
        capi.check(self.lib.fgb_serve_get_stats(self._h, ctypes.byref(s)))
        return s

    def step_latencies(self):
        cnt = ctypes.c_uint64()
        capi.check(self.lib.fgb_serve_step_latencies(self._h, None, 0, ctypes.byref(cnt)))
        buf = (ctypes.c_double * max(cnt.value, 1))()
        capi.check(self.lib.fgb_serve_step_latencies(self._h, buf, cnt.value, ctypes.byref(cnt)))
        return np.frombuffer(buf, dtype=np.float64)[:cnt.value].copy()

    def tick_particles(self):
        """Particles stepped by each tick, aligned with step_latencies()."""
        cnt = ctypes.c_uint64()
        capi.check(self.lib.fgb_serve_tick_particles(self._h, None, 0, ctypes.byref(cnt)))
        buf = (ctypes.c_uint64 * max(cnt.value, 1))()
        capi.check(self.lib.fgb_serve_tick_particles(self._h, buf, cnt.value, ctypes.byref(cnt)))
        return np.frombuffer(buf, dtype=np.uint64)[:cnt.value].copy()

    def tick_scenes(self):
        """Requests stepped by each tick, aligned with step_latencies()."""
        cnt = ctypes.c_uint64()
        capi.check(self.lib.fgb_serve_tick_scenes(self._h, None, 0, ctypes.byref(cnt)))
        buf = (ctypes.c_uint32 * max(cnt.value, 1))()
        capi.check(self.lib.fgb_serve_tick_scenes(self._h, buf, cnt.value, ctypes.byref(cnt)))
        return np.frombuffer(buf, dtype=np.uint32)[:cnt.value].copy()

    def tick_steps(self):
        """Steps each tick advanced its group by, aligned with step_latencies()."""
        cnt = ctypes.c_uint64()
        capi.check(self.lib.fgb_serve_tick_steps(self._h, None, 0, ctypes.byref(cnt)))
        buf = (ctypes.c_uint32 * max(cnt.value, 1))()
        capi.check(self.lib.fgb_serve_tick_steps(self._h, buf, cnt.value, ctypes.byref(cnt)))
        return np.frombuffer(buf, dtype=np.uint32)[:cnt.value].copy()

    def tick_starts(self):
        """Start of each tick, seconds since the server was created."""
        cnt = ctypes.c_uint64()
        capi.check(self.lib.fgb_serve_tick_starts(self._h, None, 0, ctypes.byref(cnt)))
        buf = (ctypes.c_double * max(cnt.value, 1))()
        capi.check(self.lib.fgb_serve_tick_starts(self._h, buf, cnt.value, ctypes.byref(cnt)))
        return np.frombuffer(buf, dtype=np.float64)[:cnt.value].copy()

    def close(self):
        if self._h:
            self.lib.fgb_serve_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
