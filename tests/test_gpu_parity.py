"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer work (Morton keys, sorted order, cell ranges, MC cases and triangle
counts) must be bit-exact.  Floats: after one step positions within 1e-5*h
absolute and velocities within 1e-5*h/dt (velocity is displacement over dt),
density and lambda within 1e-5 relative (lambda relative to the scene's largest
|lambda|, since it crosses zero), mesh vertices within 1e-4*h.  The kernels
evaluate the oracle's operations in the oracle's order (no contraction, explicit
fused multiply-adds on both sides, IEEE square root and division), so in practice
the floats come out bit-identical; the tolerances are the stated contract.
"""
import ctypes

import numpy as np
import pytest

from libfluid_gb300 import capi, scenes
from libfluid_gb300.solver import Batch, SphSolver

pytestmark = pytest.mark.gpu

H = 0.1
POS_TOL = 1e-5 * H
VERT_TOL = 1e-4 * H


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _sort_on_gpu(torch, keys, vals, key_bits):
    lib = capi.load()
    n = len(keys)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals.view(np.int32)).cuda()
    ok = torch.empty_like(dk)
    ov = torch.empty_like(dv)
    sb = lib.fgb_radix_sort_scratch_bytes(n)
    scratch = torch.empty(max(sb, 1), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    capi.check(lib.fgb_radix_sort_pairs_u32(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n,
                                            key_bits, scratch.data_ptr(), sb, stream))
    torch.cuda.synchronize()
    flag = scratch[sb - 256:sb - 252].cpu().numpy().view(np.uint32)[0]
    assert flag == 0, f"sort raised device error flag {flag:#x}"
    return ok.cpu().numpy().view(np.uint32), ov.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n,key_bits,kind", [
    (1, 8, "random"), (4095, 8, "random"), (4096, 24, "random"), (4097, 9, "random"),
    (100003, 30, "random"), (1 << 20, 24, "random"), (1 << 20, 32, "random"),
    (300000, 30, "dupes"), (300000, 30, "sorted"), (300000, 30, "reversed"), (262145, 1, "random"),
])
def test_radix_sort_matches_stable_argsort(torch_cuda, n, key_bits, kind):
    rng = np.random.default_rng(n + key_bits)
    hi = (1 << key_bits) if key_bits < 32 else (1 << 32)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    if kind == "dupes":
        keys = (keys % 37).astype(np.uint32)
    elif kind == "sorted":
        keys = np.sort(keys)
    elif kind == "reversed":
        keys = np.sort(keys)[::-1].copy()
    vals = np.arange(n, dtype=np.uint32)
    k, v = _sort_on_gpu(torch_cuda, keys, vals, key_bits)
    order = np.argsort(keys, kind="stable")
    assert (k == keys[order]).all()
    assert (v == order.astype(np.uint32)).all()


@pytest.mark.parametrize("n", [1, 100, 4096, 4097, 1000003, 1 << 22])
def test_exclusive_scan_matches_cumsum(torch_cuda, n):
    torch = torch_cuda
    lib = capi.load()
    rng = np.random.default_rng(n)
    x = rng.integers(0, 7, n).astype(np.uint32)
    dx = torch.from_numpy(x.view(np.int32)).cuda()
    out = torch.empty_like(dx)
    tot = torch.zeros(1, dtype=torch.int32, device="cuda")
    sb = lib.fgb_scan_scratch_bytes(n)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    capi.check(lib.fgb_exclusive_scan_u32(dx.data_ptr(), out.data_ptr(), tot.data_ptr(), n, scratch.data_ptr(), sb,
                                          torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    want = np.concatenate([[0], np.cumsum(x.astype(np.uint64))[:-1]]).astype(np.uint32)
    assert (out.cpu().numpy().view(np.uint32) == want).all()
    assert int(tot.cpu().numpy().view(np.uint32)[0]) == int(x.astype(np.uint64).sum())


def _cells_of_scene(batch, k, cells_all):
    gi = batch.grid_info(k)
    c = cells_all.reshape(-1, 2)[gi.table_offset:gi.table_offset + gi.table_size].astype(np.int64)
    first = sum(batch.counts[:k])
    occ = c[:, 1] > c[:, 0]
    c[occ] -= first
    return c.ravel().astype(np.uint32)


def _check_step(oracle_mod, params, parts, cfg, colliders=None, steps=1):
    """Each step starts both sides from the same particles (the oracle's state), so
    integers are compared bit-exact on identical input.  (Across several steps the
    GPU's rounding-level float differences may move a particle across a cell
    boundary, which changes its stale-grid neighbour set -- a property of the
    reference algorithm, not an error.)"""
    state = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(state), cfg)])
    if colliders is not None:
        batch.set_colliders(0, colliders)
    for s in range(steps):
        if s:
            batch.upload(0, state)
        ref = scenes.copy_particles(state)
        batch.step(1)
        pr = oracle_mod.step(params, cfg, ref, colliders=colliders, probe=True)
        got = batch.download(0)
        keys = batch.probe(capi.PROBE_KEYS, np.uint32)
        order = batch.probe(capi.PROBE_ORDER, np.uint32)
        cells = _cells_of_scene(batch, 0, batch.probe(capi.PROBE_CELLS, np.uint32))
        lam = batch.probe(capi.PROBE_LAMBDA, np.float32)
        rho = batch.probe(capi.PROBE_DENSITY, np.float32)
        assert batch.error_flags() == 0
        assert (order == pr["order"]).all(), "sorted order differs"
        assert (keys == pr["keys"]).all(), "Morton keys differ"
        assert (cells == pr["cells"]).all(), "cell ranges differ"
        assert (got["id"] == ref["id"]).all()
        fluid = ref["type"] == capi.TYPE_FLUID
        rel = np.abs(rho[fluid] - pr["density"][fluid]) / np.abs(pr["density"][fluid])
        assert rel.max() <= 1e-5, f"step {s}: density rel err {rel.max()}"
        lam_scale = np.abs(pr["lambda"]).max()
        assert np.abs(lam - pr["lambda"]).max() <= 1e-5 * lam_scale, "lambda differs"
        dx = np.abs(got["position"] - ref["position"]).max()
        dv = np.abs(got["velocity"] - ref["velocity"]).max()
        assert dx <= POS_TOL, f"step {s}: position max-abs {dx}"
        # velocities are (x_new - x_old) / dt, so the position tolerance becomes 1e-5 h / dt
        assert dv <= POS_TOL / cfg.dt, f"step {s}: velocity max-abs {dv}"
        assert (got["colour"] == ref["colour"]).all() and (got["type"] == ref["type"]).all()
        state = ref
    batch.close()
    solver.close()
    return got, ref


def test_step_parity_dam_break_32k(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break_32k()
    _check_step(oracle_mod, params, parts, cfg)


def test_step_parity_sphere_collider(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((24, 20, 24), (2.4, 2.0, 2.4), seed=21, sphere=(1.2, 0.3, 1.2, 0.5))
    # start the block above the sphere so that particles are projected in the first steps
    parts["position"].reshape(-1, 3)[:, 1] += 0.05
    _check_step(oracle_mod, params, parts, cfg, steps=3)


def test_step_parity_unequal_masses(oracle_mod):
    # unequal masses: the baseline's delta and vorticity-apply passes read their
    # neighbours' masses from the separate arrays (the packed copies need one mass)
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((20, 16, 20), (2.0, 2.0, 2.0), seed=151)
    parts["mass"][::7] = np.float32(1.25)
    parts["mass"][3::11] = np.float32(0.8)
    parts["type"][::19] = capi.TYPE_OBSTACLE
    _check_step(oracle_mod, params, parts, cfg, steps=3)


def test_step_parity_ref_profile_with_triangles_and_obstacles(oracle_mod):
    params = capi.params(capi.PROFILE_REF, H)
    parts, cfg = scenes.dam_break((16, 16, 16), (2.0, 2.0, 2.0), seed=31)
    parts["mass"][:] = 1.0
    parts["velocity"].reshape(-1, 3)[:, 1] = -0.5
    parts["type"][::17] = capi.TYPE_OBSTACLE
    cfg.n_wells = 1
    cfg.wells[0].centre[:] = (1.0, 1.0, 1.0)
    cfg.wells[0].force = 2.0
    cfg.constant_force[:] = (0.0, -9.8, 0.0)
    # a floor made of two triangles just above y = 0.1
    tris = np.array([[0, 0.1, 0, 2, 0.1, 0, 0, 0.1, 2], [2, 0.1, 0, 2, 0.1, 2, 0, 0.1, 2]], np.float32)
    _check_step(oracle_mod, params, parts, cfg, colliders=tris, steps=2)


def test_surface_parity_after_step(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break_32k()
    ref = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(parts, cfg)])
    batch.step(2)
    oracle_mod.step(params, cfg, ref)
    oracle_mod.step(params, cfg, ref)
    tris = batch.surface(0)
    lat = batch.probe(capi.PROBE_LATTICE, np.float32).reshape(-1, 4)
    cases = batch.probe(capi.PROBE_CUBE_CASES, np.uint8)
    otris, olat, ocol, ocases = oracle_mod.surface(params, cfg, ref, want_lattice=True)
    assert batch.error_flags() == 0
    # field: value relative to rho0; unit normals absolute, loosely -- normalising a
    # gradient that nearly cancels amplifies the ~1e-8 position differences
    assert np.abs(lat[:, 0] - olat[:, 0]).max() <= 1e-5 * params.rho0
    assert np.abs(lat[:, 1:] - olat[:, 1:]).max() <= 1e-2
    # classification and counts of the GPU lattice are bit-exact against the oracle
    # marching the very same lattice
    mtris, mcases = oracle_mod.march(params, cfg, lat.ravel(), np.zeros(len(lat), np.uint32))
    assert (cases == mcases).all()
    assert len(tris) == len(mtris)
    assert np.abs(tris[:, :18] - mtris[:, :18]).max() <= VERT_TOL
    # after two independently advanced steps a node lying within ~1e-8 of the
    # isolevel may classify differently; such cubes must be vanishingly rare
    mismatch = np.count_nonzero(cases != ocases)
    assert mismatch <= max(2, 1e-5 * len(cases)), mismatch
    assert abs(len(tris) - len(otris)) <= 4 * mismatch
    # identical particle input (the oracle's state): cases bit-exact, vertices 1e-4 h
    same = Batch(solver, [(scenes.copy_particles(ref), cfg)])
    stris = same.surface(0)
    scases = same.probe(capi.PROBE_CUBE_CASES, np.uint8)
    assert (scases == ocases).all()
    assert len(stris) == len(otris)
    assert np.abs(stris[:, :9] - otris[:, :9]).max() <= VERT_TOL
    assert np.abs(stris[:, 9:18] - otris[:, 9:18]).max() <= 1e-2
    same.close()
    batch.close()
    solver.close()


def test_surface_ref_profile_metaball(oracle_mod):
    params = capi.params(capi.PROFILE_REF, H)
    parts, cfg = scenes.dam_break((12, 12, 12), (1.5, 1.5, 1.5), seed=41)
    cfg.isolevel = 100.0
    ref = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(parts, cfg)])
    tris = batch.surface(0)
    otris, olat, _, ocases = oracle_mod.surface(params, cfg, ref, want_lattice=True)
    lat = batch.probe(capi.PROBE_LATTICE, np.float32).reshape(-1, 4)
    assert np.abs(lat[:, 0] - olat[:, 0]).max() <= 1e-5 * max(1.0, np.abs(olat[:, 0]).max())
    cases = batch.probe(capi.PROBE_CUBE_CASES, np.uint8)
    assert (cases == ocases).all()
    assert len(tris) == len(otris) > 0
    assert np.abs(tris[:, :9] - otris[:, :9]).max() <= VERT_TOL
    colours = tris[:, 18:].view(np.uint32)
    ocolours = otris[:, 18:].view(np.uint32)
    assert (colours == ocolours).all()
    batch.close()
    solver.close()


def test_surface_with_obstacles_and_colours_on_identical_input(oracle_mod):
    # obstacles are left out of the field and the colour mean; the scene is surfaced
    # straight after its upload (no step), so the obstacle count of the upload is in use
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((14, 12, 14), (1.6, 1.6, 1.6), seed=43)
    rng = np.random.default_rng(43)
    parts["colour"][:] = rng.integers(0, 1 << 32, len(parts["mass"]), dtype=np.uint64).astype(np.uint32)
    parts["type"][::7] = capi.TYPE_OBSTACLE
    ref = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(parts, cfg)])
    tris = batch.surface(0)
    otris, olat, ocol, ocases = oracle_mod.surface(params, cfg, ref, want_lattice=True)
    cases = batch.probe(capi.PROBE_CUBE_CASES, np.uint8)
    assert batch.error_flags() == 0
    assert (cases == ocases).all()
    assert len(tris) == len(otris) > 0
    assert np.abs(tris[:, :9] - otris[:, :9]).max() <= VERT_TOL
    assert (tris[:, 18:].view(np.uint32) == otris[:, 18:].view(np.uint32)).all()
    batch.close()
    solver.close()


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_surface_with_a_world_scale_on_identical_input(oracle_mod, profile):
    # world units twice the solver's: the field divides each position by the scale
    # (baseline) or scales the node (ref), and the range tests see those values
    params = capi.params(profile, H)
    parts, cfg = scenes.dam_break((14, 12, 14), (1.6, 1.6, 1.6), seed=47)
    cfg.scale = 2.0
    for a in range(3):
        cfg.min_bound[a] *= 2.0
        cfg.max_bound[a] *= 2.0
    parts["position"] *= np.float32(2.0)
    if profile == capi.PROFILE_REF:
        cfg.isolevel = 100.0
    ref = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(parts, cfg)])
    tris = batch.surface(0)
    otris, olat, ocol, ocases = oracle_mod.surface(params, cfg, ref, want_lattice=True)
    lat = batch.probe(capi.PROBE_LATTICE, np.float32).reshape(-1, 4)
    cases = batch.probe(capi.PROBE_CUBE_CASES, np.uint8)
    assert batch.error_flags() == 0
    assert np.abs(lat[:, 0] - olat[:, 0]).max() <= 1e-5 * max(params.rho0, np.abs(olat[:, 0]).max())
    assert (cases == ocases).all()
    assert len(tris) == len(otris) > 0
    assert np.abs(tris[:, :9] - otris[:, :9]).max() <= 2.0 * VERT_TOL
    assert (tris[:, 18:].view(np.uint32) == otris[:, 18:].view(np.uint32)).all()
    batch.close()
    solver.close()


def test_advance_drop_in_matches_oracle(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((20, 20, 20), (2.0, 2.0, 2.0), seed=51)
    cfg.surface = 1
    ref = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    for _ in range(3):
        mesh = solver.advance(cfg, parts)
        oracle_mod.step(params, cfg, ref)
    otris = oracle_mod.surface(params, cfg, ref)
    assert (parts["id"] == ref["id"]).all()
    assert np.abs(parts["position"] - ref["position"]).max() <= POS_TOL
    assert len(mesh) == len(otris)
    solver.close()


def test_batch_results_independent_of_composition(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    specs = [scenes.cube_scene(n, 900 + i) for i, n in enumerate([9000, 30000, 12000])]
    solver = SphSolver(params=params)
    mixed = Batch(solver, [(scenes.copy_particles(p), c) for p, c in specs])
    mixed.step(5)
    for k, (p, c) in enumerate(specs):
        alone = Batch(solver, [(scenes.copy_particles(p), c)])
        alone.step(5)
        a = alone.download(0)
        m = mixed.download(k)
        for f in ("id", "position", "velocity"):
            assert (a[f] == m[f]).all(), (k, f)
        # the surface of a scene inside the batch: same triangles, bit for bit, in the
        # same order (its cubes are classified and emitted among the other scenes')
        tris = alone.surface(0)
        assert len(tris) == mixed.surface_all()[k] > 0
        assert (mixed.surface_fetch(k).view(np.uint32) == tris.view(np.uint32)).all(), k
        alone.close()
    mixed.close()
    solver.close()


def test_ref_profile_parity_in_the_clumped_regime(oracle_mod):
    """The reference's constants clump the fluid (~100-200 candidates per particle after
    a few dozen steps): from the oracle's state after 25 steps, five more steps on a
    fresh batch -- its rows overflow the default capacities and grow, near rows come and
    go -- agree with the oracle step by step (keys, order and cells bit-exact)."""
    params = capi.params(capi.PROFILE_REF, H)
    parts, cfg = scenes.dam_break_32k()
    for _ in range(25):
        oracle_mod.step(params, cfg, parts)
    _check_step(oracle_mod, params, parts, cfg, steps=5)


def test_100_step_statistics_within_one_percent(oracle_mod):
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break_32k()
    ref = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(parts, cfg)])
    batch.step(99)
    for _ in range(99):
        oracle_mod.step(params, cfg, ref)
    batch.step(1)
    got = batch.download(0)
    rho = batch.probe(capi.PROBE_DENSITY, np.float32)
    pr = oracle_mod.step(params, cfg, ref, probe=True)
    ke_g, ke_o = scenes.kinetic_energy(got), scenes.kinetic_energy(ref)
    assert abs(ke_g - ke_o) <= 0.01 * ke_o
    com_g, com_o = scenes.centre_of_mass(got), scenes.centre_of_mass(ref)
    assert np.abs(com_g - com_o).max() <= 0.01 * np.abs(com_o).max()
    err_g = np.abs(rho / params.rho0 - 1.0)
    err_o = np.abs(pr["density"] / params.rho0 - 1.0)
    assert abs(err_g.mean() - err_o.mean()) <= 0.01 * max(err_o.mean(), 1e-3) + 1e-4
    assert abs(err_g.max() - err_o.max()) <= 0.01 * err_o.max() + 1e-3
    batch.close()
    solver.close()


def test_invalid_config_is_an_error_not_a_fault():
    params = capi.params(capi.PROFILE_BASELINE, H)
    solver = SphSolver(params=params)
    parts, cfg = scenes.dam_break((8, 8, 8), (1.0, 1.0, 1.0), seed=1)
    cfg.iterations = 0
    with pytest.raises(capi.FluidError) as e:
        Batch(solver, [(parts, cfg)])
    assert e.value.code == capi.FGB_ERR_INVALID
    cfg.iterations = 4
    cfg.scale = 0.0
    with pytest.raises(capi.FluidError):
        solver.advance(cfg, parts)
    # the context is still usable
    cfg.scale = 1.0
    solver.advance(cfg, parts)
    solver.close()


def test_autotune_changes_no_result():
    # the tuner's trial steps are ordinary steps under other launch shapes: a tuned
    # batch, an untuned one (fresh solver) and a later batch that takes the cached
    # shape all compute the same bits
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((24, 16, 24), (2.4, 2.4, 2.4), seed=61)
    tuned_solver, plain_solver = SphSolver(params=params), SphSolver(params=params)
    a = Batch(tuned_solver, [(scenes.copy_particles(parts), cfg)])
    r = a.autotune(2)
    # three CTA sizes, the four other skins, persistent tile queues of 1 and 2
    # particles per thread, then near rows with and without Verlet lists in turn
    # (five trials)
    assert r.block in (64, 128, 256) and r.trials == 14 and r.steps == 28
    assert r.persistent in (0, 1) and r.particles_per_thread in (1, 2) and r.verlet in (0, 1)
    assert any(abs(r.skin - s) < 1e-6 for s in (0.1, 0.15, 0.2, 0.25, 0.3))
    b = Batch(plain_solver, [(scenes.copy_particles(parts), cfg)])
    b.step(r.steps)
    c = Batch(tuned_solver, [(scenes.copy_particles(parts), cfg)])
    c.step(r.steps)
    ga, gb, gc = a.download(0), b.download(0), c.download(0)
    for f in ("id", "position", "velocity"):
        assert (ga[f] == gb[f]).all() and (gc[f] == gb[f]).all(), f
    for x in (a, b, c):
        x.close()
    tuned_solver.close()
    plain_solver.close()


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_near_rows_without_verlet_lists_give_the_same_bits(profile, monkeypatch):
    # FGB_VERLET=0: the first lambda pass walks and writes the near rows, later passes
    # use them or walk, and the vorticity passes walk; every sum is over the same
    # neighbours in the same order
    params = capi.params(profile, H)
    parts, cfg = scenes.dam_break((24, 16, 24), (2.4, 2.4, 2.4), seed=67)
    parts["type"][::13] = capi.TYPE_OBSTACLE
    solver = SphSolver(params=params)
    monkeypatch.setenv("FGB_VERLET", "1")
    with_lists = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    with_lists.step(12)
    monkeypatch.setenv("FGB_VERLET", "0")
    near_only = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    near_only.step(12)
    a, b = with_lists.download(0), near_only.download(0)
    for f in ("id", "position", "velocity"):
        assert (a[f] == b[f]).all(), f
    assert with_lists.error_flags() == 0 and near_only.error_flags() == 0
    with_lists.close()
    near_only.close()
    solver.close()


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_persistent_tile_queues_give_the_bits_of_flat_grids(profile, monkeypatch):
    # the gathers as persistent grids whose CTAs take tiles of 1 or 3 x blockDim
    # particles from a counter: each particle's work is unchanged, so three scenes of
    # different sizes (tiles straddle scene boundaries), with obstacles, step to the
    # same bits as with flat grids
    params = capi.params(profile, H)
    specs = []
    for k, (dims, ext) in enumerate((((25, 16, 24), 2.5), ((10, 30, 10), 1.5), ((7, 7, 7), 0.7))):
        parts, cfg = scenes.dam_break(dims, (ext, ext, ext), seed=130 + k)
        parts["type"][::11] = capi.TYPE_OBSTACLE
        specs.append((parts, cfg))
    solver = SphSolver(params=params)
    out = []
    for env in ({"FGB_PERSISTENT": "0"}, {"FGB_PERSISTENT": "1", "FGB_PPT": "1"},
                {"FGB_PERSISTENT": "1", "FGB_PPT": "3"}):
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        b = Batch(solver, [(scenes.copy_particles(p), c) for p, c in specs])
        b.step(10)
        out.append([b.download(k) for k in range(len(specs))])
        assert b.error_flags() == 0
        b.close()
        for k in env:
            monkeypatch.delenv(k)
    for run in out[1:]:
        for k in range(len(specs)):
            for f in ("id", "position", "velocity", "colour"):
                assert (run[k][f] == out[0][k][f]).all(), (k, f)
    solver.close()


@pytest.mark.parametrize("profile", [capi.PROFILE_BASELINE, capi.PROFILE_REF])
def test_packed_neighbour_reads_give_the_bits_of_separate_arrays(profile, monkeypatch):
    # the delta and vorticity-apply passes read neighbours from the lambda and
    # vorticity passes' packed copies (p* with lambda or |omega| in w) when no
    # neighbour mass is needed or every mass is equal; FGB_PACKED=0 reads the separate
    # arrays: the same bits.  (Unequal masses in the baseline profile read the separate
    # arrays either way; the oracle checks that path, test_step_parity_unequal_masses.)
    params = capi.params(profile, H)
    for masses in ("equal", "unequal"):
        parts, cfg = scenes.dam_break((20, 16, 20), (2.0, 2.0, 2.0), seed=150)
        parts["type"][::17] = capi.TYPE_OBSTACLE
        if masses == "unequal":
            parts["mass"][::7] = np.float32(1.25)
        solver = SphSolver(params=params)
        out = []
        for packed in ("1", "0"):
            monkeypatch.setenv("FGB_PACKED", packed)
            b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
            b.step(8)
            out.append(b.download(0))
            assert b.error_flags() == 0
            b.close()
        monkeypatch.delenv("FGB_PACKED")
        for f in ("position", "velocity", "colour"):
            assert (out[0][f] == out[1][f]).all(), (masses, f)
        solver.close()


def test_advance_surface_frames_do_not_change_the_state():
    # asking for a surface on some frames changes nothing in the particles: the
    # drop-in keeps its resident scene across frames that differ only in that flag
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = scenes.dam_break((16, 16, 16), (1.6, 1.6, 1.6), seed=71)
    a, b = scenes.copy_particles(parts), scenes.copy_particles(parts)
    sa, sb = SphSolver(params=params), SphSolver(params=params)
    for frame in range(6):
        cfg.surface = frame % 2
        mesh = sa.advance(cfg, a)
        assert (mesh is not None and len(mesh) > 0) == bool(frame % 2)
        cfg.surface = 0
        sb.advance(cfg, b)
    for f in ("id", "position", "velocity", "colour"):
        assert (a[f] == b[f]).all(), f
    sa.close()
    sb.close()
