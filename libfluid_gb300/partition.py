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
    fewest outstanding particle-steps (ties to the lowest rank).  A single front end
    that sees completions reports them with done(); ranks that each run a copy over
    the same request stream (route_stream) call route() alone, so that the copies
    see the same history and agree on every request with no message: the balance is
    then over the particle-steps assigned so far."""

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


def route_stream(requests, rank, world, n_of=lambda r: r[1], steps_of=lambda r: r[2]):
    """This rank's requests of a stream every rank holds in the same order: each
    request routed by a Router that is never told of completions, so every rank
    computes the same owner for every request.  Returns (position in the stream,
    request) pairs."""
    router = Router(world)
    return [(k, r) for k, r in enumerate(requests) if router.route(k, n_of(r), steps_of(r)) == rank]


def barrier():
    """A barrier over the default process group, when there is one."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def sharded_run(specs, rank, world, run_local, size_of=None):
    """The sharded form of a batch of independent scenes: this rank's share
    (local_scenes) goes to run_local(list of (global index, spec)), which returns a
    dict of host-side results; all ranks start together and the ranks' dicts are
    exchanged once at the end.  Returns every rank's dict, indexed by rank; combine()
    merges them."""
    mine = local_scenes(specs, rank, world, size_of)
    barrier()
    local = run_local(mine)
    local = dict(local, rank=rank, scenes=[i for i, _ in mine])
    return gather_summary(local)


def combine(per_rank, sum_keys=(), max_keys=(), merge_keys=(), concat_keys=()):
    """One summary of a sharded run: sum_keys added over ranks (work done), max_keys
    their maximum (the job's time is its slowest rank's), merge_keys dicts united
    (results by global index), concat_keys lists joined in rank order."""
    out = {"ranks": len(per_rank)}
    for k in sum_keys:
        out[k] = sum(r[k] for r in per_rank)
    for k in max_keys:
        out[k] = max(r[k] for r in per_rank)
    for k in merge_keys:
        m = {}
        for r in per_rank:
            m.update(r[k])
        out[k] = m
    for k in concat_keys:
        out[k] = [x for r in per_rank for x in r[k]]
    return out
