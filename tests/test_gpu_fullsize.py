"""The workloads at their full sizes on the GPU.

One step of the 1 048 576- and 8 388 608-particle dam breaks against the oracle on
identical input (integers bit-exact, floats to the stated tolerances), then
size-independent properties over longer runs: no device error flag, sorted keys
whose cell ranges cover every particle, ids a permutation, every particle inside
its box and outside the sphere collider (but where the sphere dips below the floor
and the box clamp wins), finite velocities; marching cubes of the
1M scene classified exactly as the oracle classifies the same lattice; and the 64
batched scenes bit-identical alone and inside the batch after 100 steps with
surfaces every 10.
"""
import numpy as np
import pytest

from libfluid_gb300 import capi, scenes
from libfluid_gb300.solver import Batch, SphSolver

pytestmark = pytest.mark.gpu

H = 0.1
POS_TOL = 1e-5 * H


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _one_step_parity(oracle_mod, params, parts, cfg):
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    ref = scenes.copy_particles(parts)
    batch.step(1)
    pr = oracle_mod.step(params, cfg, ref, probe=True)
    got = batch.download(0)
    assert batch.error_flags() == 0
    assert (batch.probe(capi.PROBE_ORDER, np.uint32) == pr["order"]).all()
    assert (batch.probe(capi.PROBE_KEYS, np.uint32) == pr["keys"]).all()
    assert (got["id"] == ref["id"]).all()
    assert np.abs(got["position"] - ref["position"]).max() <= POS_TOL
    assert np.abs(got["velocity"] - ref["velocity"]).max() <= POS_TOL / cfg.dt
    return solver, batch


def _invariants(batch, k, parts0, cfg):
    got = batch.download(k)
    n = len(parts0["mass"])
    assert batch.error_flags() == 0
    assert (np.sort(got["id"]) == np.sort(parts0["id"])).all()
    assert np.isclose(got["mass"].astype(np.float64).sum(), parts0["mass"].astype(np.float64).sum(), rtol=1e-12)
    p = got["position"].reshape(n, 3)
    v = got["velocity"].reshape(n, 3)
    assert np.isfinite(p).all() and np.isfinite(v).all()
    lo, hi = np.array(cfg.min_bound[:]), np.array(cfg.max_bound[:])
    assert (p >= lo - 1e-6).all() and (p <= hi + 1e-6).all()
    if cfg.sphere_enabled:
        # projected onto the sphere, then clamped to the box: only where the sphere
        # dips below the floor can the clamp put a particle back inside it
        c, r = np.array(cfg.sphere[:3]), cfg.sphere[3]
        inside = np.linalg.norm(p - c, axis=1) < r * (1 - 1e-5)
        assert (p[inside, 1] <= lo[1] + 1e-6).all()
    return got


def _keys_and_cells(batch):
    keys = batch.probe(capi.PROBE_KEYS, np.uint32)
    assert (np.diff(keys.astype(np.int64)) >= 0).all()
    gi = batch.grid_info(0)
    cells = batch.probe(capi.PROBE_CELLS, np.uint32).reshape(-1, 2)[gi.table_offset:gi.table_offset + gi.table_size]
    occ = cells[:, 1] > cells[:, 0]
    # occupied ranges tile [0, n) and every key in a range is that cell's key
    assert int((cells[occ, 1] - cells[occ, 0]).sum()) == len(keys)
    starts = cells[occ, 0]
    assert (keys[starts] == np.nonzero(occ)[0].astype(np.uint32)).all()


def test_dam_break_1m_one_step_parity_then_200_steps_and_surface(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break_1m()
    solver, batch = _one_step_parity(oracle_mod, params, parts, cfg)
    batch.step(199)
    _keys_and_cells(batch)
    _invariants(batch, 0, parts, cfg)
    tris = batch.surface(0)
    assert len(tris) > 0
    lat = batch.probe(capi.PROBE_LATTICE, np.float32)
    cases = batch.probe(capi.PROBE_CUBE_CASES, np.uint8)
    mtris, mcases = oracle_mod.march(params, cfg, lat, np.zeros(len(lat) // 4, np.uint32))
    assert (cases == mcases).all()
    assert len(mtris) == len(tris)
    batch.close()
    solver.close()


def test_double_dam_8m_one_step_parity_then_20_steps(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.double_dam_8m()
    solver, batch = _one_step_parity(oracle_mod, params, parts, cfg)
    batch.step(20)
    _keys_and_cells(batch)
    _invariants(batch, 0, parts, cfg)
    assert len(batch.surface(0)) > 0
    assert batch.error_flags() == 0
    batch.close()
    solver.close()


def test_batched_64_scenes_100_steps_match_alone():
    params = capi.params(capi.PROFILE_BASELINE, H)
    specs = scenes.batched_64()
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(p), c) for p, c in specs])
    counts = None
    for s in range(1, 101):
        batch.step(1)
        if s % 10 == 0:
            counts = batch.surface_all()
    assert batch.error_flags() == 0
    sizes = [len(p["mass"]) for p, _ in specs]
    for k in (int(np.argmin(sizes)), len(specs) // 2, int(np.argmax(sizes))):
        p, c = specs[k]
        alone = Batch(solver, [(scenes.copy_particles(p), c)])
        alone.step(100)
        a, m = alone.download(0), _invariants(batch, k, p, c)
        for f in ("id", "position", "velocity"):
            assert (a[f] == m[f]).all(), (k, f)
        assert len(alone.surface(0)) == counts[k]
        alone.close()
    batch.close()
    solver.close()
