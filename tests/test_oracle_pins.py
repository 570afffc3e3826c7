"""Pin the oracle's integer building blocks to the reference's own code.

Two sources: the committed golden vectors (tests/golden/reference_integers.json,
made by tests/golden/make_golden.py from the reference's curves.h, mctable.hpp and
mc.h), and, where the reference tree is present, the live reference shim.
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_integers.json")


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def test_morton_matches_reference_golden(oracle_lib, golden):
    L = oracle_lib.lib()
    for x, y, z, k in golden["morton"]:
        assert L.orc_morton(x, y, z) == k, (x, y, z)


def test_morton_decode_matches_reference_golden(oracle_lib, golden):
    L = oracle_lib.lib()
    for k, x, y, z in golden["decode"]:
        assert (L.orc_morton_decode(k, 0), L.orc_morton_decode(k, 1), L.orc_morton_decode(k, 2)) == (x, y, z)


def test_reference_wraps_minus_one_to_1023(oracle_lib, golden):
    # the reference's unclamped -1 becomes coordinate 1023; the oracle clamps instead,
    # and the wrapped key is exactly the key of coordinate 1023
    assert golden["morton_wrap_x_minus_1_y5_z7"] == oracle_lib.lib().orc_morton(1023, 5, 7)


def test_mc_tables_match_reference_golden(oracle_lib, golden):
    em, nv, tri = oracle_lib.mc_tables()
    assert em.tolist() == golden["edge_table"]
    assert em.tolist() == golden["cl_edge_table"]
    assert nv.tolist() == golden["num_verts"]
    assert nv.tolist() == golden["cl_num_verts"]
    ref_tri = np.array(golden["tri_table"])
    ours = tri.astype(np.int64)
    ours[ours == 255] = -1
    assert (ours == ref_tri).all()
    cl_tri = np.array(golden["cl_tri_table"])
    assert (tri.astype(np.int64) == cl_tri).all()  # OpenCL copy terminates with 255


def test_live_reference_shim_agrees(oracle_lib):
    R = oracle_lib.ref_lib()
    if R is None:
        pytest.skip("reference tree not present (oracle/_ref not built)")
    L = oracle_lib.lib()
    rng = np.random.default_rng(7)
    for x, y, z in rng.integers(0, 1024, (2000, 3)):
        assert L.orc_morton(int(x), int(y), int(z)) == R.ref_morton(int(x), int(y), int(z))
    for k in rng.integers(0, 1 << 30, 2000):
        for a in range(3):
            assert L.orc_morton_decode(int(k), a) == R.ref_morton_decode(int(k), a)
    em, nv, tri = oracle_lib.mc_tables()
    for c in range(256):
        assert em[c] == R.ref_edge_table(c) == R.ref_cl_edge_table(c)
        assert nv[c] == R.ref_num_verts(c) == R.ref_cl_num_verts(c)
        for i in range(16):
            want = R.ref_tri_table(c, i)
            assert (tri[c, i] if tri[c, i] != 255 else -1) == want
            assert tri[c, i] == R.ref_cl_tri_table(c, i)
