"""Uploads and downloads by kernels on the caller's arrays (hostio.cu) against the
pinned staging path (FGB_HOST_IO=staged): the same bytes in, the same steps, the
same bytes out -- bit-exact, on ragged sizes, with obstacles, custom ids, null
colour/id inputs and partial output views."""
import ctypes

import numpy as np
import pytest

from libfluid_gb300 import capi, scenes
from libfluid_gb300.solver import Batch, SphSolver

pytestmark = pytest.mark.gpu

H = 0.1
FIELDS = ("id", "type", "mass", "position", "velocity", "colour")


def _same(a, b):
    for f in FIELDS:
        assert a[f].shape == b[f].shape and (a[f] == b[f]).all(), f


def _batch(monkeypatch, solver, specs, staged):
    if staged:
        monkeypatch.setenv("FGB_HOST_IO", "staged")
    else:
        monkeypatch.delenv("FGB_HOST_IO", raising=False)
    b = Batch(solver, specs)
    monkeypatch.delenv("FGB_HOST_IO", raising=False)
    return b


def _require_direct(b):
    if not b.host_io_direct():
        pytest.skip("this device does not address pageable host memory")


def _scene(dims, seed):
    parts, cfg = scenes.dam_break(dims, (1.6, 1.6, 1.6), seed=seed)
    n = len(parts["mass"])
    rng = np.random.default_rng(seed)
    parts["type"][::7] = capi.TYPE_OBSTACLE
    parts["id"][:] = rng.permutation(n).astype(np.uint64) + np.uint64(1 << 40)
    parts["colour"][:] = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    return parts, cfg


@pytest.mark.parametrize("dims", [(13, 11, 7), (16, 16, 16), (1, 1, 1)])
def test_direct_and_staged_paths_give_identical_state(monkeypatch, dims):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _scene(dims, 401)
    solver = SphSolver(params=params)
    direct = _batch(monkeypatch, solver, [(scenes.copy_particles(parts), cfg)], staged=False)
    staged = _batch(monkeypatch, solver, [(scenes.copy_particles(parts), cfg)], staged=True)
    _require_direct(direct)
    assert not staged.host_io_direct()
    # an upload then a download gives the input back unchanged (no step between)
    _same(direct.download(0), parts)
    _same(staged.download(0), parts)
    direct.step(3)
    staged.step(3)
    a, b = direct.download(0), staged.download(0)
    _same(a, b)
    assert sorted(a["id"].tolist()) == sorted(parts["id"].tolist())
    assert len(direct.surface(0)) == len(staged.surface(0))
    for x in (direct, staged):
        assert x.error_flags() == 0
        x.close()
    solver.close()


def test_null_colour_and_id_inputs(monkeypatch):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _scene((12, 10, 9), 403)
    solver = SphSolver(params=params)
    outs = []
    for staged in (False, True):
        b = _batch(monkeypatch, solver, [(scenes.copy_particles(parts), cfg)], staged)
        if not staged:
            _require_direct(b)
        pv = capi.particles_view(parts)
        pv.colour = None
        pv.id = None
        capi.check(b.lib.fgb_batch_upload(b.handle, 0, ctypes.byref(pv)))
        b.step(2)
        out = b.download(0)
        assert (out["colour"] == np.uint32(0xFFFFFFFF)).all()
        assert sorted(out["id"].tolist()) == list(range(len(parts["mass"])))
        outs.append(out)
        b.close()
    _same(outs[0], outs[1])
    solver.close()


def test_partial_download_view(monkeypatch):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _scene((15, 9, 11), 405)
    solver = SphSolver(params=params)
    b = _batch(monkeypatch, solver, [(scenes.copy_particles(parts), cfg)], staged=False)
    _require_direct(b)
    b.step(2)
    full = b.download(0)
    n = len(parts["mass"])
    pos = np.full(3 * n, np.nan, np.float32)
    ids = np.zeros(n, np.uint64)
    pv = capi.Particles()
    pv.n = n
    pv.position = pos.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    pv.id = ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    capi.check(b.lib.fgb_batch_download(b.handle, 0, ctypes.byref(pv)))
    assert (pos == full["position"]).all() and (ids == full["id"]).all()
    b.close()
    solver.close()


def test_reupload_that_adds_obstacles(monkeypatch):
    """The obstacle count of a direct upload reaches the scene table: a re-upload
    with obstacles steps like a fresh batch of the same particles."""
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((14, 12, 10), (1.6, 1.6, 1.6), seed=407)
    solver = SphSolver(params=params)
    b = _batch(monkeypatch, solver, [(scenes.copy_particles(parts), cfg)], staged=False)
    _require_direct(b)
    b.step(2)
    state = b.download(0)
    state["type"][::5] = capi.TYPE_OBSTACLE
    b.upload(0, state)
    fresh = _batch(monkeypatch, solver, [(scenes.copy_particles(state), cfg)], staged=True)
    b.step(2)
    fresh.step(2)
    _same(b.download(0), fresh.download(0))
    b.close()
    fresh.close()
    solver.close()


def test_advance_direct_equals_staged(monkeypatch):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((20, 18, 17), (2.0, 2.0, 2.0), seed=409, sphere=(1.0, 0.5, 1.0, 0.3))
    cfg.surface = 1
    results = []
    for staged in (False, True):
        if staged:
            monkeypatch.setenv("FGB_HOST_IO", "staged")
        else:
            monkeypatch.delenv("FGB_HOST_IO", raising=False)
        solver = SphSolver(params=params)
        host = scenes.copy_particles(parts)
        meshes = [len(solver.advance(cfg, host)) for _ in range(3)]
        results.append((host, meshes))
        solver.close()
    monkeypatch.delenv("FGB_HOST_IO", raising=False)
    _same(results[0][0], results[1][0])
    assert results[0][1] == results[1][1]


def test_download_into_fresh_mappings(monkeypatch):
    """Output arrays on pages the host never wrote (fresh anonymous mappings) get
    every element written, as with reused arrays."""
    import mmap
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _scene((17, 13, 11), 411)
    solver = SphSolver(params=params)
    b = _batch(monkeypatch, solver, [(scenes.copy_particles(parts), cfg)], staged=False)
    _require_direct(b)
    b.step(2)
    want = b.download(0)
    n = len(parts["mass"])
    maps = []

    def fresh(count, dt):
        m = mmap.mmap(-1, count * np.dtype(dt).itemsize, flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
        maps.append(m)
        return np.frombuffer(m, dtype=dt, count=count)

    out = {"id": fresh(n, np.uint64), "type": fresh(n, np.int32), "mass": fresh(n, np.float32),
           "position": fresh(3 * n, np.float32), "velocity": fresh(3 * n, np.float32),
           "colour": fresh(n, np.uint32)}
    pv = capi.particles_view(out)
    capi.check(b.lib.fgb_batch_download(b.handle, 0, ctypes.byref(pv)))
    _same({k: np.array(v) for k, v in out.items()}, want)
    del out, pv
    b.close()
    solver.close()


def test_advance_with_null_colour_and_id(monkeypatch):
    """fgb_advance with no colour and no id arrays: both host-I/O paths give the same
    particles, in Morton order, and leave the absent arrays alone."""
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((18, 14, 16), (1.8, 1.6, 1.8), seed=413)
    outs = []
    for staged in (False, True):
        if staged:
            monkeypatch.setenv("FGB_HOST_IO", "staged")
        else:
            monkeypatch.delenv("FGB_HOST_IO", raising=False)
        solver = SphSolver(params=params)
        host = scenes.copy_particles(parts)
        for _ in range(3):
            pv = capi.particles_view(host)
            pv.colour = None
            pv.id = None
            capi.check(solver.lib.fgb_advance(solver.handle, ctypes.byref(cfg), ctypes.byref(pv), None, 0, None))
        solver.close()
        outs.append(host)
    monkeypatch.delenv("FGB_HOST_IO", raising=False)
    for f in ("type", "mass", "position", "velocity"):
        assert (outs[0][f] == outs[1][f]).all(), f
    for f in ("id", "colour"):  # untouched
        assert (outs[0][f] == parts[f]).all() and (outs[1][f] == parts[f]).all(), f


def test_advance_with_triangles_obstacles_and_surface_matches_the_batch_path(monkeypatch):
    """fgb_advance (on the direct path: split upload, obstacle count written into the
    device scene table, downloads beside and inside the step) against the same frames
    run through a batch's upload, step, surface and download, ref profile with
    triangle colliders, obstacles and a well, colliders changing between frames."""
    params = capi.params(capi.PROFILE_REF, H)
    parts, cfg = scenes.dam_break((16, 14, 16), (2.0, 2.0, 2.0), seed=417)
    parts["mass"][:] = 1.0
    parts["type"][::13] = capi.TYPE_OBSTACLE
    cfg.n_wells = 1
    cfg.wells[0].centre[:] = (1.0, 1.0, 1.0)
    cfg.wells[0].force = 2.0
    cfg.surface = 1
    floor = np.array([[0, 0.1, 0, 2, 0.1, 0, 0, 0.1, 2], [2, 0.1, 0, 2, 0.1, 2, 0, 0.1, 2]], np.float32)
    ramp = np.array([[0, 0.3, 0, 2, 0.1, 0, 0, 0.3, 2]], np.float32)
    frames = [floor, floor, ramp, None, floor]
    solver = SphSolver(params=params)
    host = scenes.copy_particles(parts)
    meshes = [solver.advance(cfg, host, colliders=c) for c in frames]
    solver.close()
    ref_solver = SphSolver(params=params)
    state = scenes.copy_particles(parts)
    want = []
    for c in frames:
        b = _batch(monkeypatch, ref_solver, [(scenes.copy_particles(state), cfg)], staged=True)
        b.set_colliders(0, c)
        b.step(1)
        want.append(b.surface(0))
        state = b.download(0)
        b.close()
    ref_solver.close()
    _same(host, state)
    for got, ref in zip(meshes, want):  # bits: the colour columns are raw ARGB words
        assert got.shape == ref.shape and (got.view(np.uint32) == ref.view(np.uint32)).all()
