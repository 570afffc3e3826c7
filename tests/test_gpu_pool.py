"""Device blocks that a solver's batches hand back are reused by its next batches
(a per-solver pool instead of cudaFree/cudaMalloc).  A block may go back while the
steps that use it are still queued on the solver's stream; the next batch's work
queues behind them, so its results equal those of a fresh solver bit for bit."""

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


def _alone(params, parts, cfg, steps):
    solver = SphSolver(params=params)
    b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    b.step(steps)
    out = b.download(0)
    b.close()
    solver.close()
    return out


def test_blocks_released_with_steps_queued_are_reused_safely():
    params = capi.params(capi.PROFILE_BASELINE, H)
    big, cb = scenes.cube_scene(110000, 31)
    small, cs = scenes.cube_scene(60000, 32)
    want = _alone(params, small, cs, 3)
    solver = SphSolver(params=params)
    for _ in range(3):
        a = Batch(solver, [(scenes.copy_particles(big), cb)])
        a.step(4)        # queued, not waited for
        a.close()        # its blocks go back to the pool while the steps run
        b = Batch(solver, [(scenes.copy_particles(small), cs)])
        b.step(3)
        _same(b.download(0), want)
        assert b.error_flags() == 0
        b.close()
    solver.close()


def test_many_create_destroy_cycles_of_mixed_sizes():
    params = capi.params(capi.PROFILE_BASELINE, H)
    specs = [scenes.cube_scene(n, 40 + i) for i, n in enumerate([4096, 30000, 13824, 50000])]
    want = [_alone(params, p, c, 2) for p, c in specs]
    solver = SphSolver(params=params)
    rng = np.random.default_rng(7)
    for _ in range(12):
        pick = sorted(rng.choice(len(specs), size=int(rng.integers(1, len(specs) + 1)), replace=False).tolist())
        b = Batch(solver, [(scenes.copy_particles(specs[k][0]), specs[k][1]) for k in pick])
        b.step(2)
        for j, k in enumerate(pick):
            _same(b.download(j), want[k])
        b.close()
    solver.close()


def test_batch_grows_within_the_pool():
    """A source that outgrows the batch's arrays re-allocates them from the pool while
    earlier steps may still be queued."""
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.cube_scene(13824, 51)
    solver = SphSolver(params=params)
    b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    b.step(2)
    n = b.sources_drains(0, [((0.6, 0.9, 0.6), (0.0, 0.0, 0.0), 20000, 9, 0xFFFFFFFF)], [])
    assert n > len(parts["mass"])
    edited = b.download(0)
    b.step(2)
    got = b.download(0)
    assert b.error_flags() == 0
    b.close()
    solver.close()
    _same(got, _alone(params, edited, cfg, 2))



def test_prepare_changes_no_result():
    """fgb_batch_prepare (graphs and scene table set up ahead of the first step)."""
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.cube_scene(30000, 71)
    solver = SphSolver(params=params)
    a = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    capi.check(b.lib.fgb_batch_prepare(b.handle))
    capi.check(b.lib.fgb_batch_prepare(b.handle))  # a second call is a no-op
    a.step(3)
    b.step(3)
    _same(a.download(0), b.download(0))
    a.close()
    b.close()
    solver.close()
