"""The C++ drop-in (include/fluid_gb300/cudasph.hpp) over the C ABI: it compiles
against the source-compatible fluid types, and on a GPU it gives the same frame
results as the C ABI called directly."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_demo.cpp")
LIBDIR = os.path.join(ROOT, "libfluid_gb300", "_build")


def _compile(tmp_path):
    from libfluid_gb300 import build
    build.build()
    exe = str(tmp_path / "adapter_demo")
    cmd = ["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), SRC,
           "-L" + LIBDIR, "-lfluidgb", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adapter_compiles_and_links(tmp_path):
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_adapter_matches_c_abi(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = json.loads(r.stdout.strip().splitlines()[-1])

    from libfluid_gb300 import capi
    from libfluid_gb300.solver import SphSolver
    ix, iy, iz = np.meshgrid(np.arange(12), np.arange(12), np.arange(12), indexing="ij")
    # the same float32 operations as the C++ program: 0.025f + 0.05f * x
    f = lambda a: np.float32(0.025) + np.float32(0.05) * a.ravel().astype(np.float32)  # noqa: E731
    pos = np.stack([f(ix), f(iy), f(iz)], 1)
    n = len(pos)
    parts = {"id": np.arange(n, dtype=np.uint64), "type": np.zeros(n, np.int32), "mass": np.ones(n, np.float32),
             "position": pos.astype(np.float32).ravel(), "velocity": np.zeros(3 * n, np.float32),
             "colour": np.full(n, 0xFF2D1010, np.uint32)}
    cfg = capi.Config()
    cfg.dt, cfg.scale, cfg.resolution, cfg.isolevel, cfg.iterations, cfg.surface = 0.0083, 1.0, 2.0, 100.0, 4, 1
    cfg.constant_force[:] = (0.0, -9.8, 0.0)
    cfg.max_bound[:] = (1.5, 1.5, 1.5)
    solver = SphSolver(profile=capi.PROFILE_REF)
    rec = capi.to_records(parts)
    for _ in range(3):
        mesh, results = solver.advance_records(cfg, rec, None, [(7, (0.3, 0.05, 0.3))])
    parts = capi.from_records(rec)
    p = parts["position"].reshape(-1, 3).astype(np.float64)
    v = parts["velocity"].reshape(-1, 3).astype(np.float64)
    sp = float((p[:, 0] + 2 * p[:, 1] + 3 * p[:, 2]).sum())
    sv = float((v[:, 0] + 2 * v[:, 1] + 3 * v[:, 2]).sum())
    assert got["n"] == n
    assert got["triangles"] == len(mesh)
    assert got["pos"] == pytest.approx(sp, rel=1e-7)
    assert got["vel"] == pytest.approx(sv, rel=1e-6, abs=1e-6)
    h = 0
    for i in parts["id"]:
        h = (h * 1000003 + int(i)) % (1 << 64)
    assert got["id_hash"] == h
    assert got["queries"] == len(results) == 1
    assert (got["q_neighbours"], got["q_colour"]) == (results[0][2], results[0][3])
    solver.close()


@pytest.mark.gpu
def test_dropin_frames_program_matches_c_abi():
    # bench.py's drop-in leg: tests/cpp/dropin_frames.cpp drives cuda::SphSolver::advance
    # on a std::vector<fluid::Particle> (baseline profile, sphere collider); its final
    # positions equal those of fgb_advance on the same scene, frame for frame
    import sys
    sys.path.insert(0, ROOT)
    import bench
    from libfluid_gb300 import capi, scenes
    from libfluid_gb300.solver import SphSolver
    parts, cfg = scenes.dam_break((24, 16, 24), (2.4, 2.0, 2.4), seed=161, sphere=(1.2, 0.3, 1.2, 0.4))
    got = bench.dropin_frames(scenes.copy_particles(parts), cfg, 2, 3)
    assert "pos_checksum" in got, got
    solver = SphSolver(params=capi.params(capi.PROFILE_BASELINE, 0.1))
    state = scenes.copy_particles(parts)
    cfg.surface = 0
    for _ in range(5):
        solver.advance(cfg, state)
    solver.close()
    p = state["position"].reshape(-1, 3).astype(np.float32).astype(np.float64)
    want = 0.0
    for x, y, z in p:  # the program's order of summation
        want += x + 2.0 * y + 3.0 * z
    assert got["n"] == len(parts["mass"])
    assert got["pos_checksum"] == pytest.approx(want, rel=1e-8)  # printed to 9 digits
