"""Sharding independent scenes across ranks (one process per GPU).

A single scene's step does not shard without a halo exchange of width h once per
solver iteration, so the single-scene path runs one replica per rank.  A batch of
independent scenes (the reference steps each of its solver instances on its own,
fluid/oclsph.hpp:289-420 per `advance` call) shards by scene: every rank computes
the same assignment from the scene sizes alone, steps its own scenes with no
collective on the data path, and only host-side summaries (counts, timings,
checksums) are exchanged once at the end.

Assignment is longest-processing-time-first over the particle count, the cost of a
scene's step being linear in it: scenes in decreasing size (ties by index) go to
the least-loaded rank (ties to the lowest rank).  Its makespan is at most 4/3 of
the optimum; the tests check the looser bound max load <= mean + largest scene.
"""
import heapq


def assign(sizes, world):
    """Scene indices per rank (each list ascending) for scenes of the given sizes."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [sorted(o) for o in out]


def loads(sizes, parts):
    return [sum(int(sizes[i]) for i in p) for p in parts]


def local_scenes(specs, rank, world, size_of=None):
    """(global index, spec) pairs of this rank's share of `specs`.  size_of(spec)
    gives a scene's particle count (default: len(spec[0]["mass"]))."""
    size_of = size_of or (lambda s: len(s[0]["mass"]))
    parts = assign([size_of(s) for s in specs], world)
    return [(i, specs[i]) for i in parts[rank]]


class Router:
    """Serving front end over `world` ranks: a request goes to the rank with the
    fewest outstanding particle-steps (ties to the lowest rank).  Every rank can run
    the same router over the same request stream and reach the same routing, so no
    message is needed to agree on it."""

    def __init__(self, world):
        self.outstanding = [0] * world
        self.owner = {}

    def route(self, ticket, n, steps):
        r = min(range(len(self.outstanding)), key=lambda k: (self.outstanding[k], k))
        self.outstanding[r] += int(n) * int(steps)
        self.owner[ticket] = (r, int(n) * int(steps))
        return r

    def done(self, ticket):
        r, work = self.owner.pop(ticket)
        self.outstanding[r] -= work
        return r


def gather_summary(obj):
    """All ranks' host-side summaries (a list indexed by rank) over the default
    process group; the one exchange of a sharded run, after the timed work."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out
