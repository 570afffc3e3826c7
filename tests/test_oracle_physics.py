"""Physics checks of the baseline profile's velocity terms (XSPH viscosity and
vorticity confinement, PBF paper eq. 15-17), which have no counterpart in the
reference to pin them: properties of the continuum operators that the SPH
estimates must keep.  They run on the oracle; the GPU gives the oracle's bits
(tests/test_gpu_parity.py)."""
import numpy as np
import pytest

from libfluid_gb300 import capi, scenes

H = 0.1


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


def _cube():
    parts, cfg = scenes.cube_scene(13824, 5)
    cfg.constant_force[:] = (0.0, 0.0, 0.0)
    return parts, cfg


def _rotate(parts, omega):
    """v = omega y-hat x (x - c): a rigid rotation about the cube's vertical axis."""
    p = parts["position"].reshape(-1, 3)
    c = (p.min(0) + p.max(0)) / 2
    v = np.zeros_like(p)
    v[:, 0] = omega * (p[:, 2] - c[2])
    v[:, 2] = -omega * (p[:, 0] - c[0])
    parts["velocity"][:] = v.astype(np.float32).ravel()
    return c


def test_vorticity_of_a_rigid_rotation_is_twice_its_angular_velocity(orc):
    # curl(omega x r) = 2 omega: in the cube's interior the SPH estimate points along
    # +y with magnitude ~2 omega (scaled by the local density over rest density)
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _cube()
    _rotate(parts, 0.5)
    p = parts["position"].reshape(-1, 3)
    lo, hi = p.min(0), p.max(0)
    pr = orc.step(params, cfg, scenes.copy_particles(parts), probe=True)
    om = pr["omega"].reshape(-1, 4)
    ps = p[pr["order"]]
    inner = np.all((ps > lo + 2.5 * H) & (ps < hi - 2.5 * H), axis=1)
    assert inner.sum() > 1000
    mean = om[inner, :3].mean(0)
    assert 0.85 < mean[1] / 1.0 < 1.15, mean
    assert abs(mean[0]) < 0.02 and abs(mean[2]) < 0.02, mean


def test_uniform_motion_changes_nothing_else(orc):
    # Galilean invariance: the same cube moving at a uniform velocity u steps like the
    # cube at rest, shifted by u dt (XSPH and vorticity see only velocity differences)
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _cube()
    cfg.min_bound[:] = (-1.0, -1.0, -1.0)
    cfg.max_bound[:] = (3.0, 3.0, 3.0)
    rest = scenes.copy_particles(parts)
    moving = scenes.copy_particles(parts)
    u = np.array([0.3, -0.2, 0.1], np.float32)
    moving["velocity"][:] = np.tile(u, len(moving["mass"]))
    orc.step(params, cfg, rest)
    orc.step(params, cfg, moving)
    ia, ib = np.argsort(rest["id"]), np.argsort(moving["id"])
    dp = moving["position"].reshape(-1, 3)[ib] - rest["position"].reshape(-1, 3)[ia]
    dv = moving["velocity"].reshape(-1, 3)[ib] - rest["velocity"].reshape(-1, 3)[ia]
    assert np.abs(dp - u * np.float32(cfg.dt) * np.float32(cfg.scale)).max() < 1e-5 * H
    assert np.abs(dv - u).max() < 2e-3


def test_vorticity_confinement_feeds_the_rotation(orc):
    # the confinement force eps (N x omega), N along grad |omega|, restores rotation:
    # a vortex whose angular velocity peaks on its axis (|omega| largest at the core)
    # keeps more angular momentum about the axis the larger eps is
    params = capi.params(capi.PROFILE_BASELINE, H)
    parts, cfg = _cube()
    p = parts["position"].reshape(-1, 3)
    c = (p.min(0) + p.max(0)) / 2
    r = p - c
    w = 2.0 * np.exp(-((r[:, 0] ** 2 + r[:, 2] ** 2) / 0.25 ** 2))
    v = np.zeros_like(p)
    v[:, 0] = w * r[:, 2]
    v[:, 2] = -w * r[:, 0]
    parts["velocity"][:] = v.astype(np.float32).ravel()
    ang = []
    for eps in (0.0, params.vorticity_epsilon * 50, params.vorticity_epsilon * 200):
        pe = capi.params(capi.PROFILE_BASELINE, H)
        pe.vorticity_epsilon = eps
        q = scenes.copy_particles(parts)
        orc.step(pe, cfg, q)
        x = q["position"].reshape(-1, 3) - c
        vq = q["velocity"].reshape(-1, 3)
        ang.append(float((x[:, 2] * vq[:, 0] - x[:, 0] * vq[:, 2]).sum()))  # L_y
    assert 0 < ang[0] < ang[1] < ang[2], ang


def test_xsph_smooths_velocity_noise(orc):
    # XSPH adds c sum m_b/rho0 (v_b - v_a) W_ab: a smoothing of the velocity field, so
    # noise on a cube at rest leaves the step with less velocity variance the larger c is
    parts, cfg = _cube()
    rng = np.random.default_rng(3)
    parts["velocity"][:] = (0.05 * rng.standard_normal(parts["velocity"].shape)).astype(np.float32)
    var = []
    for c in (0.0, 0.05, 0.2):
        pc = capi.params(capi.PROFILE_BASELINE, H)
        pc.xsph_c = c
        pc.vorticity_epsilon = 0.0
        q = scenes.copy_particles(parts)
        orc.step(pc, cfg, q)
        v = q["velocity"].reshape(-1, 3).astype(np.float64)
        var.append(float(((v - v.mean(0)) ** 2).sum(1).mean()))
    assert var[0] > var[1] > var[2], var
