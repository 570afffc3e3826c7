"""Packed record streams: the C packers against an independent numpy restatement
of the reference's packed layout (samples/structures.hpp particleDef /
meshTriangleDef / headerDef over mmf::writer::writePacked), and on a GPU the
device-packed streams of a resident scene against the host packers."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from libfluid_gb300 import capi, scenes, wire


@pytest.fixture(scope="module")
def lib():
    from libfluid_gb300 import build
    build.build()
    return capi.load()


def test_record_sizes_match_the_reference_layout(lib):
    # id 8 + type 4 + mass 4 + colour 4 + position 12 + velocity 12
    assert wire.PARTICLE.itemsize == 44
    # v0..v2 36 + n0..n2 36 + c (3 x u32) 12
    assert wire.TRIANGLE.itemsize == 84 == ctypes.sizeof(capi.MeshTriangle)
    # id 8 + point 12 + neighbours 8 + averageColour 4
    assert wire.QUERY.itemsize == 32
    assert wire.HEADER.itemsize == 24


def _numpy_particles(parts):
    n = len(parts["mass"])
    recs = np.zeros(n, wire.PARTICLE)
    recs["id"] = parts["id"]
    recs["type"] = parts["type"]
    recs["mass"] = parts["mass"]
    recs["colour"] = parts["colour"]
    recs["position"] = parts["position"].reshape(-1, 3)
    recs["velocity"] = parts["velocity"].reshape(-1, 3)
    return recs


def test_particle_stream_matches_numpy_packing(lib):
    parts, _ = scenes.dam_break((6, 5, 4), (1.0, 1.0, 1.0), seed=3)
    rng = np.random.default_rng(3)
    n = len(parts["mass"])
    parts["id"][:] = rng.integers(0, 1 << 63, n, dtype=np.uint64)
    parts["colour"][:] = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    parts["velocity"][:] = rng.standard_normal(3 * n).astype(np.float32)
    parts["type"][::5] = capi.TYPE_OBSTACLE
    buf = wire.particles(parts, timestamp_ms=1234567890123, lib=lib)
    assert len(buf) == 24 + 44 * n
    h, recs = wire.read(buf, wire.PARTICLE)
    assert (int(h["timestamp"]), int(h["entries"]), int(h["written"])) == (1234567890123, n, n)
    assert recs.tobytes() == _numpy_particles(parts).tobytes()


def test_triangle_stream_is_the_records_verbatim(lib):
    rng = np.random.default_rng(5)
    tris = rng.standard_normal((37, 21)).astype(np.float32)
    tris[:, 18:] = rng.integers(0, 1 << 32, (37, 3), dtype=np.uint64).astype(np.uint32).view(np.float32)
    buf = wire.triangles(tris, timestamp_ms=7, lib=lib)
    h, recs = wire.read(buf, wire.TRIANGLE)
    assert int(h["entries"]) == int(h["written"]) == 37
    assert recs.tobytes() == tris.tobytes()
    assert (recs["c"] == tris[:, 18:].view(np.uint32)).all()
    assert np.array_equal(recs["v"].reshape(-1, 9), tris[:, :9])


def test_empty_streams_and_capacity_errors(lib):
    empty = {k: v[:0] for k, v in scenes.dam_break((2, 2, 2), (1.0, 1.0, 1.0), seed=1)[0].items()}
    buf = wire.particles(empty, timestamp_ms=0, lib=lib)
    assert len(buf) == 24
    assert int(wire.read(buf, wire.PARTICLE)[0]["entries"]) == 0
    assert len(wire.triangles(np.zeros((0, 21), np.float32), lib=lib)) == 24
    parts, _ = scenes.dam_break((2, 2, 2), (1.0, 1.0, 1.0), seed=1)
    pv = capi.particles_view(parts)
    small = bytearray(24 + 44 * 8 - 1)
    size = ctypes.c_uint64()
    rc = lib.fgb_wire_particles(ctypes.byref(pv), 0, (ctypes.c_char * len(small)).from_buffer(small), len(small),
                                ctypes.byref(size))
    assert rc == capi.FGB_ERR_INVALID and size.value == 24 + 44 * 8


def test_query_stream_layout():
    buf = wire.queries([(3, (1.0, 2.0, 3.0), 17, 0xFF102030)], timestamp_ms=5)
    h, recs = wire.read(buf, wire.QUERY)
    assert int(h["entries"]) == 1 and len(buf) == 24 + 32
    assert int(recs[0]["id"]) == 3 and int(recs[0]["neighbours"]) == 17
    assert int(recs[0]["average_colour"]) == 0xFF102030


@pytest.mark.gpu
def test_device_packed_streams_match_host_packers(lib):
    from libfluid_gb300.solver import Batch, SphSolver
    params = capi.params(capi.PROFILE_BASELINE, 0.1)
    specs = [scenes.cube_scene(n, 60 + i) for i, n in enumerate([4096, 13824])]
    for k, (p, _) in enumerate(specs):
        p["id"][:] = np.arange(len(p["mass"]), dtype=np.uint64) * 7 + 1000 * k
    solver = SphSolver(params=params)
    batch = Batch(solver, [(scenes.copy_particles(p), c) for p, c in specs])
    batch.step(3)
    counts = batch.surface_all()
    for k in range(len(specs)):
        dev = wire.batch_particles(batch, k, timestamp_ms=11)
        host = wire.particles(batch.download(k), timestamp_ms=11, lib=lib)
        assert dev == host
        sdev = wire.batch_surface(batch, k, timestamp_ms=12)
        shost = wire.triangles(batch.surface_fetch(k), timestamp_ms=12, lib=lib)
        assert sdev == shost
        assert int(wire.read(sdev, wire.TRIANGLE)[0]["entries"]) == counts[k]
    batch.close()
    solver.close()


def test_cpp_header_writers_match_the_c_abi(lib, tmp_path):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "libfluid_gb300", "_build")
    exe = str(tmp_path / "wire_demo")
    r = subprocess.run(["g++", "-std=c++14", "-O2", "-Wall", "-Werror", "-I" + os.path.join(root, "include"),
                        os.path.join(root, "tests", "cpp", "wire_demo.cpp"), "-L" + libdir, "-lfluidgb",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    # three streams: 50 particles, 9 triangles, 1 query
    assert r.stdout.split() == ["ok", str(24 + 44 * 50), str(24 + 84 * 9), str(24 + 32)]
