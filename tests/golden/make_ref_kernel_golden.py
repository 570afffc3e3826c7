"""Writes tests/golden/reference_kernels.npz: what the reference's own kernels
(oracle/ref_kernels.cpp, compiled from the reference tree by oracle/Makefile)
compute on the small scene of tests/test_oracle_ref_kernels.py, so that the oracle
stays pinned to them where the reference tree is absent.

Run here, where the reference tree exists:  python tests/golden/make_ref_kernel_golden.py
Contents: the scene's digest; without triangles (4 solver iterations) and with the
triangle floor (1 iteration): sorted keys and the reference's positions,
velocities, lambda and colours after one step; then the reference's marching-cubes
lattice of the step's result (samples with a value only), cube triangle counts and
triangles.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from libfluid_gb300 import capi  # noqa: E402
from oracle import oracle  # noqa: E402

import test_oracle_ref_kernels as T  # noqa: E402


def main():
    oracle.build()
    K = oracle.ref_kernels()
    if K is None:
        sys.exit("oracle/_ref/libref_kernels.so missing: the reference tree is needed")
    params = capi.params(capi.PROFILE_REF, T.H)
    out = {}
    for with_tris in (False, True):
        parts, cfg, tris = T.golden_scene()
        out["digest"] = np.array(T.scene_digest(parts))
        tag = "t_" if with_tris else ""
        if with_tris:
            cfg.iterations = 1
        else:
            tris = None
        inputs, pr, parts = T.solve_inputs(oracle, params, cfg, parts, tris)
        ref = oracle.ref_solve(K, cfg, colliders=tris, **inputs)
        out[tag + "keys"] = pr["keys"]
        for k in ("position", "velocity", "lambda", "colour"):
            out[tag + "ref_" + k] = ref[k]
        if not with_tris:
            lat, lcol, counts, rtris = oracle.ref_surface(K, params, cfg, parts)
            idx = np.nonzero(lat[:, 0])[0].astype(np.uint32)
            out["samples"] = np.array(len(lat))
            out["lat_index"] = idx
            out["lat_value"] = lat[idx]
            out["lat_colour"] = lcol[idx]
            assert counts.max() < 256
            out["counts"] = counts.astype(np.uint8)
            out["tris"] = rtris
    path = os.path.join(HERE, "reference_kernels.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
