"""The drop-in on the caller's own particle records, and the frame's cell queries.

fgb_advance_records reads and writes an array of records in place (the layout of
fluid::Particle<size_t, float>, as the C++ adapter passes its std::vector), and must
give the bits fgb_advance gives on the same particles as separate arrays.  Its cell
queries (include/fluid/oclsph.hpp:770-791) are checked against a numpy restatement
on the oracle's grid of the same step: the fluid particles in each query point's
cell of the predicted-position grid and the truncated float mean of their colours
before the step's diffusion, results only for cells that hold fluid.
"""
import numpy as np
import pytest

from libfluid_gb300 import capi, scenes
from libfluid_gb300.solver import Batch, SphSolver

pytestmark = pytest.mark.gpu

H = 0.1


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


def _scene(profile):
    parts, cfg = scenes.dam_break((20, 16, 20), (2.0, 2.0, 2.0), seed=77)
    n = len(parts["mass"])
    rng = np.random.default_rng(77)
    parts["colour"][:] = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    parts["type"][::13] = capi.TYPE_OBSTACLE
    parts["id"][:] = rng.permutation(n).astype(np.uint64) + 1000
    if profile == capi.PROFILE_REF:
        cfg.isolevel = 100.0
    return parts, cfg


def _queries(parts, cfg):
    p = parts["position"].reshape(-1, 3)
    pts = [tuple(p[0]), tuple(p[len(p) // 2]), tuple(p[-1] + 0.01),
           (1.9, 1.9, 1.9),                                 # an empty cell inside the grid
           tuple(np.array(cfg.max_bound[:]) + 0.15),          # the grid's last cells
           (-5.0, 0.5, 0.5), (0.5, 50.0, 0.5)]              # outside the grid
    return [(100 + i, pt) for i, pt in enumerate(pts)]


def _numpy_queries(orc, params, cfg, before, pr, queries):
    """oclsph.hpp:770-791 on the oracle's grid of the step."""
    g = orc.grid(params, cfg)
    L = orc.lib()
    order, cells = pr["order"], pr["cells"].reshape(-1, 2)
    type_s, col_s = before["type"][order], before["colour"][order]
    table_n = int(L.orc_morton(*g.ext))
    out = []
    for qid, pt in queries:
        c = []
        for a in range(3):
            v = np.float32(pt[a]) / np.float32(cfg.scale)
            u = (np.float32(v) - np.float32(g.min_ext[a])) / np.float32(params.h)
            if not (u >= 0) or u >= np.float32(g.ext[a]) + 1:
                c = None
                break
            c.append(int(u))
        if c is None:
            continue
        key = int(L.orc_morton(*c))
        if key + 1 >= table_n:
            continue
        s, e = cells[key]
        sel = [i for i in range(s, e) if type_s[i] == capi.TYPE_FLUID]
        if not sel:
            continue
        sums = [0, 0, 0, 0]
        for i in sel:
            for ch in range(4):
                sums[ch] += int((int(col_s[i]) >> (24 - 8 * ch)) & 0xFF)
        argb = 0
        for ch in range(4):
            argb |= (int(np.float32(sums[ch]) / np.float32(len(sel))) & 0xFF) << (24 - 8 * ch)
        out.append((qid, len(sel), argb))
    return out


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_records_match_arrays_and_queries_match_numpy(orc, profile):
    params = capi.params(profile, H)
    parts, cfg = _scene(profile)
    tris = np.array([[0, 0.05, 0, 2, 0.05, 0, 0, 0.05, 2]], np.float32) if profile == capi.PROFILE_REF else None
    soa = scenes.copy_particles(parts)
    rec = capi.to_records(parts)
    sa, sb = SphSolver(params=params), SphSolver(params=params)
    for frame in range(3):
        before = capi.from_records(rec)
        queries = _queries(before, cfg)
        cfg.surface = frame % 2
        mesh_a = sa.advance(cfg, soa, tris)
        mesh_b, results = sb.advance_records(cfg, rec, tris, queries)
        got = capi.from_records(rec)
        for f in ("id", "type", "mass", "position", "velocity", "colour"):
            assert (got[f] == soa[f]).all(), (frame, f)
        if cfg.surface:
            # bit patterns: a degenerate normal is NaN on both paths
            assert mesh_a.shape == mesh_b.shape
            diff = np.argwhere(mesh_a.view(np.uint32) != mesh_b.view(np.uint32))
            assert len(diff) == 0, (frame, diff[:8], mesh_a[diff[:4, 0]], mesh_b[diff[:4, 0]])
        # the queries against the oracle's grid of the same step
        pr = orc.step(params, cfg, scenes.copy_particles(before), colliders=tris, probe=True)
        want = _numpy_queries(orc, params, cfg, before, pr, queries)
        assert [(q, n, c) for q, _, n, c in results] == want, frame
        # the first two points lie on particles; the rest may fall in empty cells
        assert len(want) >= 2 and all(n > 0 for _, n, _ in want)
    cfg.surface = 0
    sa.close()
    sb.close()


def test_batch_query_after_a_step_and_refused_after_a_surface(orc):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _scene(capi.PROFILE_BASELINE)
    before = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    queries = _queries(before, cfg)
    with pytest.raises(capi.FluidError):
        b.query(0, queries)  # no step yet
    b.step(1)
    got = b.query(0, queries)
    pr = orc.step(params, cfg, scenes.copy_particles(before), probe=True)
    assert [(q, n, c) for q, _, n, c in got] == _numpy_queries(orc, params, cfg, before, pr, queries)
    b.surface(0)
    with pytest.raises(capi.FluidError) as e:
        b.query(0, queries)
    assert e.value.code == capi.FGB_ERR_INVALID
    b.close()
    solver.close()


def test_staged_records_match_direct_records(monkeypatch):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _scene(capi.PROFILE_BASELINE)
    direct = capi.to_records(parts)
    sd = SphSolver(params=params)
    sd.advance_records(cfg, direct)
    monkeypatch.setenv("FGB_HOST_IO", "staged")
    staged = capi.to_records(parts)
    ss = SphSolver(params=params)
    _, res_s = ss.advance_records(cfg, staged, None, _queries(parts, cfg))
    monkeypatch.delenv("FGB_HOST_IO")
    assert (direct.view(np.uint8) == staged.view(np.uint8)).all()
    assert len(res_s) >= 3
    sd.close()
    ss.close()


def test_bad_record_layouts_are_refused():
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _scene(capi.PROFILE_BASELINE)
    rec = capi.to_records(parts)
    solver = SphSolver(params=params)
    lib = solver.lib
    for field, value in (("stride", 46), ("stride", 256), ("position", 2), ("mass", -1), ("velocity", 40)):
        rv = capi.records_view(rec)
        setattr(rv, field, value)
        rc = lib.fgb_advance_records(solver.handle, cfg, rv, None, 0, None, 0, None, None, None)
        assert rc == capi.FGB_ERR_INVALID, field
    solver.close()
