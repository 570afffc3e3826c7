"""Generate the golden vectors that pin the oracle's integer building blocks.

Run where the reference tree and oracle/_ref are present:
    make -C oracle && python tests/golden/make_golden.py
It evaluates the REFERENCE's own code (curves.h Morton encode/decode, mctable.hpp
and mc.h tables, compiled by oracle/Makefile into oracle/_ref/libref_shim.so) and
writes tests/golden/reference_integers.json.  Nothing here is computed by the
code under test.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle  # noqa: E402


def main():
    R = oracle.ref_lib()
    if R is None:
        raise SystemExit("oracle/_ref/libref_shim.so missing: run make -C oracle where the reference exists")
    rng = np.random.default_rng(20261203)
    coords = [(x, y, z) for x in range(8) for y in range(8) for z in range(8)]
    coords += [tuple(int(v) for v in rng.integers(0, 1024, 3)) for _ in range(512)]
    coords += [(1023, 1023, 1023), (1023, 0, 0), (0, 1023, 0), (0, 0, 1023), (512, 256, 128),
               (132, 68, 68), (260, 132, 132), (36, 20, 20)]
    morton = [[x, y, z, int(R.ref_morton(x, y, z))] for (x, y, z) in coords]
    # x = -1 as size_t: the reference wraps it to coordinate 1023 (curves.h:57-70)
    wrap = int(R.ref_morton((1 << 64) - 1, 5, 7))
    decode = []
    for k in [int(v) for v in rng.integers(0, 1 << 30, 256)] + [0, (1 << 30) - 1]:
        decode.append([k, int(R.ref_morton_decode(k, 0)), int(R.ref_morton_decode(k, 1)),
                       int(R.ref_morton_decode(k, 2))])
    edge = [int(R.ref_edge_table(c)) for c in range(256)]
    nverts = [int(R.ref_num_verts(c)) for c in range(256)]
    tri = [[int(R.ref_tri_table(c, i)) for i in range(16)] for c in range(256)]
    cl_edge = [int(R.ref_cl_edge_table(c)) for c in range(256)]
    cl_nverts = [int(R.ref_cl_num_verts(c)) for c in range(256)]
    cl_tri = [[int(R.ref_cl_tri_table(c, i)) for i in range(16)] for c in range(256)]
    out = {
        "source": "tom91136/libfluid include/fluid/curves.h:29-72, mctable.hpp:7,44,305, mc.h:8,44,305",
        "morton": morton,
        "morton_wrap_x_minus_1_y5_z7": wrap,
        "decode": decode,
        "edge_table": edge,
        "num_verts": nverts,
        "tri_table": tri,
        "cl_edge_table": cl_edge,
        "cl_num_verts": cl_nverts,
        "cl_tri_table": cl_tri,
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_integers.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
