"""Row capacities grow on demand: when more than 1% of a step's particles overflow
their Verlet or hit rows (and fall back to the 27-cell walk), the batch enlarges
the rows by half before its next step and the solver remembers the capacities for
the size bucket.  Growth changes no result: the state equals that of rows large
enough from the start, bit for bit."""
import ctypes
import os

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


def _overflow(b):
    n = b.counts[0]
    cnt = np.zeros(n, np.uint16)
    capi.check(b.lib.fgb_batch_probe(b.handle, capi.PROBE_LIST_COUNT, cnt.ctypes.data_as(ctypes.c_void_p), 2 * n))
    return float(np.mean(cnt == 0xFFFF))


def _run(params, parts, cfg, caps, steps):
    # lists every step (the list policy would stop building them in violent steps,
    # which leaves no rows to grow)
    env = {"FGB_LIST_CAP": str(caps[0]), "FGB_HIT_CAP": str(caps[1])} if caps else {}
    env["FGB_LIST_POLICY"] = "0"
    env["FGB_VERLET"] = "1"  # the Verlet rows are what grows
    os.environ.update(env)
    try:
        solver = SphSolver(params=params)
        b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    finally:
        for k in env:
            del os.environ[k]
    over = []
    for _ in range(steps):
        b.step(1)
        over.append(_overflow(b))
    out = b.download(0)
    assert b.error_flags() == 0
    b.close()
    solver.close()
    return out, over


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_rows_grow_from_small_capacities_without_changing_results(profile):
    params = capi.params(profile, H)
    parts, cfg = scenes.dam_break((20, 16, 20), (2.0, 1.6, 2.0), seed=91, sphere=(1.0, 0.3, 1.0, 0.3))
    grown, over = _run(params, parts, cfg, (8, 8), 12)
    assert over[0] > 0.5             # 8 entries: nearly every row overflows at first
    assert over[-1] < 0.02           # and the rows have grown past the neighbour counts
    roomy, _ = _run(params, parts, cfg, (512, 512), 12)
    _same(grown, roomy)


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_list_policy_changes_no_result(profile):
    # the list policy stops building Verlet lists and near rows when too few particles
    # of a step could use them: every pass then walks its cells, and walking scenes try
    # lists again when calm or every 8 steps.  Asked to keep lists only where 95% of a
    # pass could use them, a dam break onto a sphere switches between the two; the
    # state equals that with lists built every step, bit for bit.
    params = capi.params(profile, H)
    parts, cfg = scenes.dam_break((20, 16, 20), (2.0, 1.6, 2.0), seed=93, sphere=(1.0, 0.3, 1.0, 0.3))
    out = {}
    for policy in ("1", "0"):
        # with Verlet lists, whose marks tell the steps that built none
        os.environ.update(FGB_LIST_POLICY=policy, FGB_LIST_MIN_USE="95", FGB_VERLET="1")
        try:
            solver = SphSolver(params=params)
            b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
        finally:
            del os.environ["FGB_LIST_POLICY"], os.environ["FGB_LIST_MIN_USE"], os.environ["FGB_VERLET"]
        off = 0
        for _ in range(40):
            b.step(1)
            off += _overflow(b) == 1.0  # every row marked: no lists this step
        out[policy] = (b.download(0), off)
        assert b.error_flags() == 0
        b.close()
        solver.close()
    assert out["1"][1] > 0 and out["0"][1] == 0
    _same(out["1"][0], out["0"][0])
