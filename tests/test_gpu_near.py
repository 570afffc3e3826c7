"""Near rows (the build pass's hit row kept at h + a small skin, iterated directly by
the later lambda passes while the displacement bound holds) change no result: the
state after several steps equals that with near rows off, bit for bit, in both
physics profiles, with obstacles and a sphere collider."""
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


def _run(params, parts, cfg, skin, steps=6):
    """State after `steps` steps with near skin `skin` (fraction of h), and the largest
    fraction of particles whose last lambda pass ran over the near row."""
    import os
    os.environ["FGB_NEAR_SKIN"] = skin
    try:
        solver = SphSolver(params=params)
        b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    finally:
        del os.environ["FGB_NEAR_SKIN"]
    frac = 0.0
    for _ in range(steps):
        b.step(1)
        n = b.counts[0]
        flags = np.zeros(n, np.uint8)
        capi.check(b.lib.fgb_batch_probe(b.handle, capi.PROBE_NEAR_ROW, flags.ctypes.data_as(ctypes.c_void_p), n))
        frac = max(frac, float(flags.mean()))
    out = b.download(0)
    assert b.error_flags() == 0
    b.close()
    solver.close()
    return out, frac


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_near_rows_change_no_result_with_obstacles_and_sphere(profile):
    params = capi.params(profile, H)
    parts, cfg = scenes.dam_break((24, 20, 22), (2.4, 2.0, 2.4), seed=61, sphere=(1.2, 0.3, 1.2, 0.4))
    parts["type"][::13] = capi.TYPE_OBSTACLE
    base, used = _run(params, parts, cfg, "0")
    assert used == 0.0
    for skin in ("0.05", "0.2"):
        _same(base, _run(params, parts, cfg, skin)[0])


def test_near_rows_taken_in_a_quiet_scene():
    # baseline profile: the reference constants correct positions more per
    # iteration, so their passes seldom stay within the near skin
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.cube_scene(32768, 63)
    base, _ = _run(params, parts, cfg, "0", steps=8)
    near, used = _run(params, parts, cfg, "0.05", steps=8)
    assert used > 0.2
    _same(base, near)
