"""Sources and drains of resident scenes on the device (fgb_batch_sources_drains)
against a numpy restatement of the reference's CPU pass (oclsph.hpp:675-708):
emitted particles appended in source order (x outer, z inner), then every fluid
particle closer than a drain's width to its centre erased with the survivors'
order kept.  Bit-exact, and the next steps equal those of the edited particles
uploaded afresh."""
import numpy as np
import pytest

from libfluid_gb300 import capi, scenes
from libfluid_gb300.solver import Batch, SphSolver

pytestmark = pytest.mark.gpu

H = 0.1
FIELDS = ("id", "type", "mass", "position", "velocity", "colour")


def _apply_reference(parts, cfg, sources, drains):
    f32 = np.float32
    spacing = f32(f32(H) * f32(cfg.scale)) / f32(2)
    new = {k: [] for k in FIELDS}
    for centre, vel, rate, tag, colour in sources:
        size = f32(np.sqrt(np.float64(rate)))
        width, depth = int(np.floor(size)), int(np.ceil(size))
        off = [f32(centre[0]) - (f32(width) / f32(2)) * spacing, f32(centre[1]) - (f32(0) / f32(2)) * spacing,
               f32(centre[2]) - (f32(depth) / f32(2)) * spacing]
        for x in range(width):
            for z in range(depth):
                pos = [off[0] + f32(x) * spacing, off[1] + f32(0) * spacing, off[2] + f32(z) * spacing]
                new["id"].append(tag)
                new["type"].append(capi.TYPE_FLUID)
                new["mass"].append(1.0)
                new["position"].extend(pos)
                new["velocity"].extend(vel)
                new["colour"].append(colour)
    out = {k: np.concatenate([parts[k], np.array(new[k], parts[k].dtype)]) for k in FIELDS}
    n = len(out["mass"])
    p = out["position"].reshape(n, 3)
    keep = np.ones(n, bool)
    for centre, width in drains:
        d = np.asarray(centre, np.float32) - p
        dist = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        keep &= ~((dist < np.float32(width)) & (out["type"] != capi.TYPE_OBSTACLE))
    res = {}
    for k in FIELDS:
        v = out[k]
        res[k] = (v.reshape(n, 3)[keep].ravel() if k in ("position", "velocity") else v[keep]).copy()
    return res


def _same(a, b):
    for f in FIELDS:
        assert a[f].shape == b[f].shape and (a[f] == b[f]).all(), f


SOURCES = [((0.5, 1.0, 0.6), (0.0, -1.0, 0.5), 10, 7001, 0xFF0000FF),
           ((1.0, 1.2, 1.0), (0.2, 0.0, 0.0), 16, 7002, 0xFF00FF00)]
DRAINS = [((0.4, 0.2, 0.4), 0.25), ((1.05, 1.2, 1.05), 0.06)]


def test_single_scene_edit_matches_reference_and_steps_on_identically():
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((14, 12, 14), (1.6, 1.6, 1.6), seed=81)
    parts["type"][::11] = capi.TYPE_OBSTACLE  # obstacles are never drained
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    batch.step(3)
    before = batch.download(0)
    want = _apply_reference(before, cfg, SOURCES, DRAINS)
    assert len(want["mass"]) != len(before["mass"])  # the edit drains and emits
    count = batch.sources_drains(0, SOURCES, DRAINS)
    assert count == len(want["mass"])
    _same(batch.download(0), want)
    # two more steps equal the edited particles uploaded into a fresh batch
    fresh = Batch(solver, [(want, cfg)])
    batch.step(2)
    fresh.step(2)
    assert batch.error_flags() == 0
    _same(batch.download(0), fresh.download(0))
    assert len(batch.surface(0)) == len(fresh.surface(0))
    batch.close()
    fresh.close()
    solver.close()


def test_edit_of_one_scene_leaves_the_others_and_grows_the_batch():
    params = capi.params(capi.PROFILE_BASELINE, H)
    specs = [scenes.cube_scene(n, 90 + i) for i, n in enumerate([4096, 13824, 4096])]
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(p), c) for p, c in specs])
    batch.step(2)
    before = [batch.download(k) for k in range(3)]
    # a large source on the middle scene: the batch outgrows its arrays
    _, c1 = specs[1]
    big = [((0.6, 0.9, 0.6), (0.0, 0.0, 0.0), 20000, 9, 0xFFFFFFFF)]
    drain = [((0.3, 0.2, 0.3), 0.2)]
    want = _apply_reference(before[1], c1, big, drain)
    assert batch.sources_drains(1, big, drain) == len(want["mass"])
    _same(batch.download(0), before[0])
    _same(batch.download(1), want)
    _same(batch.download(2), before[2])
    # each scene steps on as it would alone
    batch.step(2)
    assert batch.error_flags() == 0
    for k, start in enumerate([before[0], want, before[2]]):
        alone = Batch(solver, [(start, specs[k][1])])
        alone.step(2)
        _same(batch.download(k), alone.download(0))
        alone.close()
    batch.close()
    solver.close()


def test_edit_without_sources_or_drains_changes_nothing():
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((8, 8, 8), (1.0, 1.0, 1.0), seed=83)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    batch.step(1)
    before = batch.download(0)
    assert batch.sources_drains(0) == len(before["mass"])
    _same(batch.download(0), before)
    batch.close()
    solver.close()
