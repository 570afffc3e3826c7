"""Scene sharding across ranks: the assignment, the serving router, and a
world_size-2 gloo run in which each rank steps its own scenes with the oracle and
only checksums are exchanged at the end (the GPU path shards the same way)."""
import hashlib
import json
import multiprocessing as mp
import os
import socket

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


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        specs = _specs()
        mine = partition.local_scenes(specs, rank, world)
        digests = _step_all(mine)
        everything = partition.gather_summary({"rank": rank, "scenes": [i for i, _ in mine], "digests": digests})
        if rank == 0:
            with open(out_path, "w") as f:
                json.dump(everything, f)
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
        ranks = json.load(f)
    assert [r["rank"] for r in ranks] == [0, 1]
    owned = sorted(i for r in ranks for i in r["scenes"])
    assert owned == list(range(len(SCENE_TARGETS)))
    assert all(r["scenes"] for r in ranks)  # both ranks got work
    sharded = {int(k): v for r in ranks for k, v in r["digests"].items()}
    single = _step_all(list(enumerate(_specs())))
    assert sharded == single
