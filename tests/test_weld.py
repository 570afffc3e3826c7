"""Vertex welding: the oracle's sort-based restatement against a first-appearance
dictionary (the reference's std::map walk, geometry.hpp:152-166), and on a GPU the
hash-table kernels against the oracle, bit for bit."""
import numpy as np
import pytest

from libfluid_gb300 import capi, scenes


def _python_weld(tris):
    """geometry::indexVBO2 as written: vertices in order, exact byte match reuses."""
    seen, idx, verts = {}, [], []
    for t in tris:
        for k in range(3):
            p = t[3 * k:3 * k + 3]
            key = p.tobytes()
            if key not in seen:
                seen[key] = len(verts)
                verts.append(p)
            idx.append(seen[key])
    return np.array(idx, np.uint32), np.array(verts, np.float32).reshape(-1, 3)


def _soup(n, distinct, seed):
    """n triangles whose vertices come from `distinct` positions (plus both signed
    zeros, which are different bytes and so different vertices)."""
    rng = np.random.default_rng(seed)
    pool = rng.standard_normal((distinct, 3)).astype(np.float32)
    pool[0] = (0.0, 0.0, 0.0)
    pool[1] = (-0.0, 0.0, 0.0)
    tris = np.zeros((n, 21), np.float32)
    tris[:, :9] = pool[rng.integers(0, distinct, 3 * n)].reshape(n, 9)
    tris[:, 9:18] = rng.standard_normal((n, 9)).astype(np.float32)
    return tris


@pytest.mark.parametrize("n,distinct", [(0, 2), (1, 2), (500, 40), (3000, 5000)])
def test_oracle_weld_matches_first_appearance(oracle_lib, n, distinct):
    tris = _soup(n, distinct, n + distinct)
    idx, verts = oracle_lib.weld(tris)
    pidx, pverts = _python_weld(tris)
    assert (idx == pidx).all()
    assert verts.tobytes() == pverts.tobytes()
    if n:
        assert (verts[idx].reshape(n, 9) == tris[:, :9]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("n,distinct", [(1, 2), (1000, 50), (200000, 150000), (300000, 10)])
def test_gpu_weld_matches_oracle(oracle_lib, n, distinct):
    from libfluid_gb300.weld import weld
    tris = _soup(n, distinct, 7 * n + distinct)
    idx, verts = weld(tris)
    oidx, overts = oracle_lib.weld(tris)
    assert (idx == oidx).all()
    assert verts.tobytes() == overts.tobytes()


@pytest.mark.gpu
def test_gpu_weld_of_a_resident_surface(oracle_lib):
    from libfluid_gb300.solver import Batch, SphSolver
    from libfluid_gb300.weld import batch_weld, weld
    params = capi.params(capi.PROFILE_BASELINE, 0.1)
    specs = [scenes.cube_scene(n, 80 + i) for i, n in enumerate([4096, 13824])]
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(p), c) for p, c in specs])
    batch.step(2)
    counts = batch.surface_all()
    for k in range(len(specs)):
        tris = batch.surface_fetch(k)
        idx, verts = batch_weld(batch, k, counts[k])
        oidx, overts = oracle_lib.weld(tris)
        assert (idx == oidx).all() and verts.tobytes() == overts.tobytes()
        hidx, hverts = weld(tris)  # the same triangles through the host-memory entry point
        assert (hidx == idx).all() and hverts.tobytes() == verts.tobytes()
        # triangles of a marching-cubes surface share vertices
        assert 0 < len(verts) < len(idx)
    batch.close()
    solver.close()
