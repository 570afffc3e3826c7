"""Colour diffusion of the ref profile (oclsph_kernel.h:281-303): the oracle's C
restatement against an independent numpy restatement on the oracle's own grid, and
(on a GPU) the CUDA kernels against the oracle, bit for bit."""
import numpy as np
import pytest

from libfluid_gb300 import capi, scenes

H = 0.1


def _scene(seed=41):
    params = capi.params(capi.PROFILE_REF, H)
    parts, cfg = scenes.dam_break((12, 10, 12), (1.2, 1.2, 1.2), seed=seed)
    rng = np.random.default_rng(seed)
    n = len(parts["mass"])
    parts["colour"][:] = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    parts["colour"][:16] = 0x00000000  # channels at 0: the clamp to 8 lifts them
    parts["colour"][16:32] = 0xFFFFFFFF
    parts["type"][::13] = capi.TYPE_OBSTACLE
    parts["mass"][:] = 1.0
    cfg.dt = 0.25  # a large dt/750 so that the pull toward the mean moves whole steps
    cfg.iterations = 1
    return params, parts, cfg


def _numpy_diffusion(oracle, params, cfg, colour_sorted, type_sorted, keys, cells):
    """oclsph_kernel.h:281-303 in numpy float32: 27-cell candidates (clamped to the
    grid), fluid only, itself included; mix, clamp to [8, 255], truncate."""
    g = oracle.grid(params, cfg)
    lib = oracle.lib()
    cells = cells.reshape(-1, 2)
    out = colour_sorted.copy()
    t = np.float32(cfg.dt) / np.float32(750.0)
    fluid = type_sorted != capi.TYPE_OBSTACLE
    chans = np.stack([(colour_sorted >> (8 * c)) & 0xFF for c in range(4)], 1).astype(np.int64)
    for i in np.nonzero(fluid)[0]:
        cx, cy, cz = (lib.orc_morton_decode(int(keys[i]), a) for a in range(3))
        tot = np.zeros(4, np.int64)
        cnt = 0
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    x, y, z = cx + dx, cy + dy, cz + dz
                    if not (0 <= x <= g.ext[0] and 0 <= y <= g.ext[1] and 0 <= z <= g.ext[2]):
                        continue
                    s, e = cells[lib.orc_morton(x, y, z)]
                    sel = fluid[s:e]
                    tot += chans[s:e][sel].sum(0)
                    cnt += int(sel.sum())
        v = 0
        for c in range(4):
            xo = np.float32(chans[i, c])
            ym = (np.float32(tot[c]) / np.float32(cnt)) * np.float32(1.33)
            o = xo + (ym - xo) * t
            o = min(max(o, np.float32(8.0)), np.float32(255.0))
            v |= int(o) << (8 * c)
        out[i] = v
    return out


def test_oracle_diffusion_matches_numpy_restatement(oracle_lib):
    params, parts, cfg = _scene()
    colour_in = parts["colour"].copy()
    type_in = parts["type"].copy()
    pr = oracle_lib.step(params, cfg, parts, probe=True)
    order = pr["order"]
    want = _numpy_diffusion(oracle_lib, params, cfg, colour_in[order], type_in[order], pr["keys"], pr["cells"])
    assert (parts["colour"] == want).all()
    fluid = parts["type"] == capi.TYPE_FLUID
    changed = (parts["colour"] != colour_in[order])[fluid].mean()
    assert changed > 0.5  # the scene exercises the diffusion
    assert (parts["colour"][~fluid] == colour_in[order][~fluid]).all()  # obstacles keep theirs


def test_baseline_profile_keeps_colours(oracle_lib):
    params, parts, cfg = _scene()
    params = capi.params(capi.PROFILE_BASELINE, H)
    colour_in = parts["colour"].copy()
    pr = oracle_lib.step(params, cfg, parts, probe=True)
    assert (parts["colour"] == colour_in[pr["order"]]).all()


@pytest.mark.gpu
def test_gpu_diffusion_matches_oracle(oracle_lib):
    from libfluid_gb300.solver import Batch, SphSolver
    params, parts, cfg = _scene()
    ref = scenes.copy_particles(parts)
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    for _ in range(2):
        batch.upload(0, ref)
        batch.step(1)
        oracle_lib.step(params, cfg, ref)
        got = batch.download(0)
        assert batch.error_flags() == 0
        assert (got["id"] == ref["id"]).all()
        assert (got["colour"] == ref["colour"]).all()
    batch.close()
    solver.close()
