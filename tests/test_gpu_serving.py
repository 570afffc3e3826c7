"""Serving loop on the GPU: requests of different sizes and step counts arriving
while others run are admitted, batched and finished; each result is identical to
the same scene advanced alone, and to the one-at-a-time loop."""
import time

import numpy as np
import pytest

from libfluid_gb300 import capi, scenes
from libfluid_gb300.serve import Server
from libfluid_gb300.solver import Batch, SphSolver

pytestmark = pytest.mark.gpu


def _requests():
    out = []
    for i, (n, steps, mesh) in enumerate([(9000, 7, True), (30000, 4, False), (12000, 9, True),
                                           (5000, 3, False), (20000, 6, True)]):
        parts, cfg = scenes.cube_scene(n, 700 + i)
        out.append((parts, cfg, steps, mesh))
    return out


def _alone(solver, parts, cfg, steps, mesh):
    b = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    b.step(steps)
    got = b.download(0)
    tris = b.surface(0) if mesh else None
    b.close()
    return got, tris


def _serve(solver, reqs, one_at_a_time=False, stagger=0.0, tick_particles=0, max_steps_per_tick=1):
    sv = Server(solver, budget_bytes=8 << 30, one_at_a_time=one_at_a_time, tick_particles=tick_particles,
                max_steps_per_tick=max_steps_per_tick)
    tickets = []
    for parts, cfg, steps, mesh in reqs:
        tickets.append(sv.submit(cfg, parts, steps, mesh))
        if stagger:
            time.sleep(stagger)  # later requests arrive while earlier ones run
    sv.drain(300)
    results = [sv.fetch(t) for t in tickets]
    st = sv.stats()
    lat = sv.step_latencies()
    # per-tick particles and start times line up with the latencies
    tp, t0, ks = sv.tick_particles(), sv.tick_starts(), sv.tick_steps()
    assert len(tp) == len(lat) == len(t0) == len(ks) == st.ticks
    assert int((tp * ks).sum()) == st.particle_steps
    assert ks.min() >= 1 and ks.max() <= (1 if one_at_a_time else max_steps_per_tick or 16)
    assert (np.diff(t0) >= 0).all() and (t0 >= 0).all()
    if tick_particles:
        sizes = [len(p["mass"]) for p, _, _, _ in reqs]
        assert int(tp.max()) <= max(tick_particles, max(sizes))
    sv.close()
    return results, st, lat, ks


def test_each_result_is_the_same_alone_and_in_the_mix():
    solver = SphSolver(params=capi.params(capi.PROFILE_BASELINE, 0.1))
    reqs = _requests()
    mixed, st, lat, _ = _serve(solver, reqs, stagger=0.002)
    assert st.completed == len(reqs) and st.failed == 0 and st.rejected == 0
    assert st.ticks >= max(r[2] for r in reqs)
    assert len(lat) == st.ticks
    # continuous batching: fewer ticks than running the requests back to back
    assert st.ticks < sum(r[2] for r in reqs)
    for (parts, cfg, steps, mesh), (got, tris) in zip(reqs, mixed):
        ref, rtris = _alone(solver, parts, cfg, steps, mesh)
        for f in ("id", "position", "velocity", "colour"):
            assert (got[f] == ref[f]).all(), f
        if mesh:
            assert len(tris) == len(rtris) and (tris == rtris).all()
    serial, st1, _, _ = _serve(solver, reqs, one_at_a_time=True)
    assert st1.ticks == sum(r[2] for r in reqs)
    for (got, tris), (got1, tris1) in zip(mixed, serial):
        assert (got["position"] == got1["position"]).all()
    solver.close()


def test_tick_groups_bound_the_work_per_tick_and_keep_results():
    # 32 000 particles per tick: the 32 768-particle scene runs alone, the others
    # share groups; every result still equals the scene advanced alone
    solver = SphSolver(params=capi.params(capi.PROFILE_BASELINE, 0.1))
    reqs = _requests()
    grouped, st, lat, _ = _serve(solver, reqs, stagger=0.002, tick_particles=32000)
    assert st.completed == len(reqs) and st.failed == 0
    sizes = [len(p["mass"]) for p, _, _, _ in reqs]
    work = sum(n * steps for n, (_, _, steps, _) in zip(sizes, reqs))
    assert st.particle_steps == work
    assert st.ticks >= work / max(32000, max(sizes))
    for (parts, cfg, steps, mesh), (got, tris) in zip(reqs, grouped):
        ref, rtris = _alone(solver, parts, cfg, steps, mesh)
        for f in ("id", "position", "velocity", "colour"):
            assert (got[f] == ref[f]).all(), f
        if mesh:
            assert len(tris) == len(rtris) and (tris == rtris).all()
    solver.close()


def test_small_groups_take_several_steps_a_tick_and_keep_results():
    # a 400 000-particle tick budget: groups far below half of it advance several
    # steps per tick (at most 4 here), never past a scene's last step; every result
    # equals the scene advanced alone and the particle-steps add up
    solver = SphSolver(params=capi.params(capi.PROFILE_BASELINE, 0.1))
    reqs = _requests()
    res, st, lat, ks = _serve(solver, reqs, stagger=0.002, tick_particles=400000, max_steps_per_tick=4)
    assert st.completed == len(reqs) and st.failed == 0
    sizes = [len(p["mass"]) for p, _, _, _ in reqs]
    assert st.particle_steps == sum(n * steps for n, (_, _, steps, _) in zip(sizes, reqs))
    assert ks.max() > 1
    assert st.ticks < sum(r[2] for r in reqs)
    for (parts, cfg, steps, mesh), (got, tris) in zip(reqs, res):
        ref, rtris = _alone(solver, parts, cfg, steps, mesh)
        for f in ("id", "position", "velocity", "colour"):
            assert (got[f] == ref[f]).all(), f
        if mesh:
            assert len(tris) == len(rtris) and (tris == rtris).all()
    solver.close()


def test_over_budget_request_is_rejected_and_others_complete():
    solver = SphSolver(params=capi.params(capi.PROFILE_BASELINE, 0.1))
    big, cfg = scenes.cube_scene(262144, 1)
    small, cfg2 = scenes.cube_scene(8000, 2)
    sv = Server(solver, budget_bytes=64 << 20)  # 64 MiB: the big scene can never fit
    t_big = sv.submit(cfg, big, 2)
    t_small = sv.submit(cfg2, small, 2)
    sv.drain(120)
    assert sv.poll(t_big).status == -capi.FGB_ERR_BUDGET
    assert sv.poll(t_small).status == capi.SERVE_DONE
    got, _ = sv.fetch(t_small)
    ref, _ = _alone(solver, small, cfg2, 2, False)
    assert (got["position"] == ref["position"]).all()
    with pytest.raises(capi.FluidError):
        sv.fetch(t_big)
    sv.close()
    solver.close()


def test_groups_spread_evenly_and_scenes_move_between_batches():
    """Many small scenes under a small tick budget: lightest-fit placement and the
    re-spread move resident scenes between group batches on the device; every result
    still equals the scene advanced alone."""
    solver = SphSolver(params=capi.params(capi.PROFILE_BASELINE, 0.1))
    reqs = []
    for i, (n, steps) in enumerate([(13824, 9), (4096, 3), (13824, 12), (8000, 5), (4096, 8), (13824, 4),
                                    (8000, 10), (4096, 6)]):
        parts, cfg = scenes.cube_scene(n, 800 + i)
        reqs.append((parts, cfg, steps, False))
    res, st, lat, _ = _serve(solver, reqs, stagger=0.001, tick_particles=30000)
    assert st.completed == len(reqs) and st.failed == 0
    assert st.rebuilds > 0
    for (parts, cfg, steps, _), (got, _) in zip(reqs, res):
        ref, _ = _alone(solver, parts, cfg, steps, False)
        for f in ("id", "position", "velocity", "colour"):
            assert (got[f] == ref[f]).all(), f
    solver.close()
