"""Scene sharding across ranks: the assignment, the serving router, and a
world_size-2 gloo run of the host path bench.py's sharded legs take
(partition.sharded_run and combine for the batched leg, route_stream for the
serving leg) in which each rank steps its own scenes with the oracle and only
summaries are exchanged at the end."""
import hashlib
import json
import multiprocessing as mp
import os
import socket
import time

import numpy as np
import pytest

from libfluid_gb300 import capi, partition, scenes

SCENE_TARGETS = [512, 4096, 512, 13824, 512]
STEPS = 2


def _specs():
    return [scenes.cube_scene(n, 900 + i) for i, n in enumerate(SCENE_TARGETS)]


def _digest(parts):
    h = hashlib.sha256()
    for k in ("position", "velocity", "id"):
        h.update(np.ascontiguousarray(parts[k]).tobytes())
    return h.hexdigest()


def _step_all(indexed_specs):
    from oracle import oracle
    params = capi.default_params()
    out = {}
    for i, (p, c) in indexed_specs:
        q = scenes.copy_particles(p)
        for _ in range(STEPS):
            oracle.step(params, c, q)
        out[i] = _digest(q)
    return out


def test_assign_covers_each_scene_once():
    rng = np.random.default_rng(11)
    for world in (1, 2, 3, 8):
        sizes = rng.integers(1, 10_000, size=37)
        parts = partition.assign(sizes, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        assert all(p == sorted(p) for p in parts)
        ld = partition.loads(sizes, parts)
        assert max(ld) <= sum(ld) / world + max(sizes)
        assert parts == partition.assign(list(sizes), world)  # deterministic


def test_assign_edge_cases():
    assert partition.assign([], 2) == [[], []]
    assert partition.assign([5], 3) == [[0], [], []]
    # equal sizes: ties go to the lower index and the lower rank
    assert partition.assign([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        partition.assign([1], 0)


def test_router_balances_and_is_deterministic():
    reqs = [(t, n, s) for t, (n, s) in enumerate([(4096, 100), (512, 20), (13824, 50), (512, 200), (4096, 30)])]
    a, b = partition.Router(2), partition.Router(2)
    ra = [a.route(*r) for r in reqs]
    rb = [b.route(*r) for r in reqs]
    assert ra == rb
    assert ra[0] == 0 and ra[1] == 1
    for t, _, _ in reqs:
        a.done(t)
    assert a.outstanding == [0, 0]


def test_gather_summary_without_process_group():
    assert partition.gather_summary({"x": 1}) == [{"x": 1}]


def test_combine_and_route_stream_single_rank():
    per_rank = [{"w": 2, "t": 1.5, "d": {0: "a"}, "l": [1]}, {"w": 3, "t": 0.5, "d": {3: "b"}, "l": [2, 3]}]
    c = partition.combine(per_rank, sum_keys=("w",), max_keys=("t",), merge_keys=("d",), concat_keys=("l",))
    assert c == {"ranks": 2, "w": 5, "t": 1.5, "d": {0: "a", 3: "b"}, "l": [1, 2, 3]}
    stream = [(0.0, 100, 10), (0.1, 50, 10), (0.2, 400, 1), (0.3, 10, 10)]
    assert partition.route_stream(stream, 0, 1) == list(enumerate(stream))
    r0, r1 = partition.route_stream(stream, 0, 2), partition.route_stream(stream, 1, 2)
    # particle-steps 1000, 500, 400, 100: the first to rank 0, the rest fill rank 1 up to 1000
    assert [k for k, _ in r0] == [0] and [k for k, _ in r1] == [1, 2, 3]


def _run_local(mine):
    """A rank's share of the batch, as bench.py's batched leg runs it but with the
    oracle for the GPU: results by global scene index, work done, time taken."""
    t0 = time.perf_counter()
    digests = _step_all(mine)
    return {"digests": digests, "particles": sum(len(p["mass"]) for _, (p, _) in mine),
            "seconds": time.perf_counter() - t0}


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # the batched leg's host path: sharded_run, then combine on every rank
        per_rank = partition.sharded_run(_specs(), rank, world, _run_local)
        combined = partition.combine(per_rank, sum_keys=("particles",), max_keys=("seconds",),
                                     merge_keys=("digests",))
        # the serving leg's host path: a replicated router over the same stream
        stream = scenes.serving_stream(40, 1.0, seed=3)
        routed = partition.gather_summary([k for k, _ in partition.route_stream(stream, rank, world)])
        if rank == 0:
            with open(out_path, "w") as f:
                json.dump({"ranks": [{"rank": r["rank"], "scenes": r["scenes"]} for r in per_rank],
                           "digests": combined["digests"], "particles": combined["particles"],
                           "seconds": combined["seconds"], "routed": routed}, f)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_sharded_batch_matches_single_process(tmp_path):
    pytest.importorskip("torch.distributed")
    from oracle import oracle
    oracle.build()
    out = str(tmp_path / "ranks.json")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    with open(out) as f:
        got = json.load(f)
    ranks = got["ranks"]
    assert [r["rank"] for r in ranks] == [0, 1]
    owned = sorted(i for r in ranks for i in r["scenes"])
    assert owned == list(range(len(SCENE_TARGETS)))
    assert all(r["scenes"] for r in ranks)  # both ranks got work
    specs = _specs()
    assert got["particles"] == sum(len(p["mass"]) for p, _ in specs)
    assert got["seconds"] > 0
    sharded = {int(k): v for k, v in got["digests"].items()}
    single = _step_all(list(enumerate(specs)))
    assert sharded == single
    # every request served by exactly one rank, as a single process routes them
    stream = scenes.serving_stream(40, 1.0, seed=3)
    routed = got["routed"]
    assert sorted(k for r in routed for k in r) == list(range(40))
    assert routed == [[k for k, _ in partition.route_stream(stream, r, 2)] for r in range(2)]
    assert all(routed)
