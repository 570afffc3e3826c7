"""Seeded synthetic dam-break scenes for the five workloads.

No dataset is involved: every input is generated here from a splitmix64 stream so
that Python, the CUDA library and the CPU oracle see identical particles.  The
block layout follows the reference demo's makeCube (samples/main.cpp:36-56):
particles on a cubic lattice of the given spacing; here each sits at the centre
of its lattice cell, plus a uniform jitter of +-0.005 per axis.

Workloads (h = 0.1, rho0 = 1000, mass 0.125, g = -9.81 y, dt = 1/120, 4 iterations):
  dam_break_32k      32 768 = 32^3 block in [0,3.2]x[0,1.6]^2                     seed 1
  dam_break_1m       1 048 576 = 128x64x128 block in [0,12.8]x[0,6.4]^2,
                     static sphere r=1 at (8,0.8,3.2)                               seed 2
  double_dam_8m      8 388 608: two 128x128x256 blocks at both x ends of
                     [0,25.6]x[0,12.8]^2                                            seed 3
  batched_64         64 scenes, n log-uniform in [8192, 262144], cube side rounded
                     to a multiple of 8, box 2x block in x and 1.5x in y, z         seed 4
  serving stream     Poisson arrivals; n log-uniform in [16384, 2097152], steps
                     uniform in [20, 200], 50% request a mesh                       seed 5
"""
import math

import numpy as np

from . import capi

SPACING = 0.05
JITTER = 0.005
MASS = 0.125
COLOUR = 0xFF2D1010  # the reference demo's particle colour (samples/main.cpp:50)
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed, count):
    """count outputs of splitmix64 seeded with `seed` (vectorised)."""
    with np.errstate(over="ignore"):
        i = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed, count):
    """Uniform floats in [0, 1) with 24 random bits (exact in float32)."""
    z = splitmix64(seed, count)
    return ((z >> np.uint64(40)).astype(np.float64) / float(1 << 24))


def block(dims, origin, seed, id_offset=0):
    """Particles of a dims=(nx,ny,nz) block at `origin` (x slowest, z fastest)."""
    nx, ny, nz = dims
    n = nx * ny * nz
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    lattice = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    jit = (uniform(seed, 3 * n).reshape(n, 3) * 2.0 - 1.0) * JITTER
    pos = np.asarray(origin, np.float64) + (lattice + 0.5) * SPACING + jit
    return {
        "id": np.arange(id_offset, id_offset + n, dtype=np.uint64),
        "type": np.zeros(n, np.int32),
        "mass": np.full(n, MASS, np.float32),
        "position": pos.astype(np.float32).ravel(),
        "velocity": np.zeros(3 * n, np.float32),
        "colour": np.full(n, COLOUR, np.uint32),
    }


def concat(parts):
    return {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}


def config(min_bound, max_bound, sphere=None, iterations=4, surface=0,
           profile=capi.PROFILE_BASELINE):
    c = capi.Config()
    c.dt = 1.0 / 120.0
    c.scale = 1.0
    c.resolution = 2.0
    c.isolevel = 500.0
    c.iterations = iterations
    c.surface = surface
    c.constant_force[:] = (0.0, -9.81, 0.0)
    c.min_bound[:] = min_bound
    c.max_bound[:] = max_bound
    if sphere is not None:
        c.sphere_enabled = 1
        c.sphere[:] = sphere
    if profile == capi.PROFILE_REF:
        c.isolevel = 100.0
    return c


def dam_break(side_dims, box, seed, sphere=None, iterations=4):
    parts = block(side_dims, (0.0, 0.0, 0.0), seed)
    return parts, config((0.0, 0.0, 0.0), box, sphere, iterations)


def dam_break_32k(iterations=4):
    return dam_break((32, 32, 32), (3.2, 1.6, 1.6), 1, iterations=iterations)


def dam_break_1m(iterations=4):
    return dam_break((128, 64, 128), (12.8, 6.4, 6.4), 2, sphere=(8.0, 0.8, 3.2, 1.0),
                     iterations=iterations)


def double_dam_8m(iterations=4):
    a = block((128, 128, 256), (0.0, 0.0, 0.0), 3)
    b = block((128, 128, 256), (19.2, 0.0, 0.0), 3 * 1000003, id_offset=len(a["mass"]))
    return concat([a, b]), config((0.0, 0.0, 0.0), (25.6, 12.8, 12.8), iterations=iterations)


def cube_side(n_target):
    """Cube side (particles) of the batched/serving recipe: the cube root of n rounded
    to the nearest multiple of 8 (halves round up), at least 8."""
    return max(8, int(math.floor(n_target ** (1.0 / 3.0) / 8.0 + 0.5)) * 8)


def cube_scene(n_target, seed, iterations=4):
    """A scene of the batched/serving recipe: cube side = cbrt(n) rounded to a
    multiple of 8; box 2x the block extent in x, 1.5x in y and z."""
    side = cube_side(n_target)
    ext = side * SPACING
    parts = block((side, side, side), (0.0, 0.0, 0.0), seed)
    return parts, config((0.0, 0.0, 0.0), (2.0 * ext, 1.5 * ext, 1.5 * ext), iterations=iterations)


def batched_sizes(count=64, seed=4, lo=8192, hi=262144):
    u = uniform(seed, count)
    n = np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))
    return [int(v) for v in n]


def batched_64(iterations=4, count=64):
    sizes = batched_sizes(count)
    return [cube_scene(n, 4 * 7919 + i, iterations) for i, n in enumerate(sizes)]


def serving_stream(count, rate_hz, seed=5, lo=16384, hi=2097152):
    """Request list (arrival time s, n, steps, want_mesh, scene seed)."""
    u = uniform(seed, 4 * count).reshape(count, 4)
    gaps = -np.log(1.0 - u[:, 0]) / rate_hz
    t = np.cumsum(gaps)
    n = np.exp(np.log(lo) + u[:, 1] * (np.log(hi) - np.log(lo)))
    steps = 20 + np.floor(u[:, 2] * 181).astype(np.int64)
    mesh = (u[:, 3] < 0.5).astype(np.int64)
    out = []
    for i in range(count):
        side = cube_side(n[i])
        out.append((float(t[i]), side ** 3, int(steps[i]), int(mesh[i]), 5 * 104729 + i))
    return out


def realised_count(n_target):
    side = cube_side(n_target)
    return side ** 3


def copy_particles(p):
    return {k: v.copy() for k, v in p.items()}


def kinetic_energy(p):
    v = p["velocity"].reshape(-1, 3).astype(np.float64)
    return float(0.5 * np.sum(p["mass"].astype(np.float64) * np.sum(v * v, axis=1)))


def centre_of_mass(p):
    x = p["position"].reshape(-1, 3).astype(np.float64)
    m = p["mass"].astype(np.float64)
    return (m[:, None] * x).sum(axis=0) / m.sum()


def fmt_bytes(b):
    for unit in ("B", "KB", "MB", "GB"):
        if b < 1024:
            return f"{b:.1f}{unit}"
        b /= 1024
    return f"{b:.1f}TB"


__all__ = [n for n in dir() if not n.startswith("_") and n not in ("math", "np", "capi")]
