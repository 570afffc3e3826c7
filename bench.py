#!/usr/bin/env python
"""Benchmark: PBF particle-steps/s (4 solver iterations) on one GB300.

Default workload: dam_break_1m -- 1 048 576 particles (128x64x128 block, spacing
0.05, seeded jitter) in [0,12.8]x[0,6.4]^2 with a static sphere r=1 at
(8,0.8,3.2); h=0.1, rho0=1000, mass 0.125, dt=1/120, 4 iterations, s_corr, XSPH,
vorticity; FP32.  A "step" is one PBF step of the whole scene.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value      whole-job particle-steps/s, state resident in HBM, L2 flushed (a
           256 MiB write) before every timed step, each step timed with CUDA
           events on the launching stream, max over ranks.
e2e        the same metric through fgb_advance (the reference-facing C ABI call)
           with host arrays: upload, step and write-back every step.
roofline   the dominant kernel's algorithmic bytes per launch over its mean
           CUDA-event duration, against the measured HBM copy bandwidth; beside
           it ("issue") the same kernel's warp instructions per launch (from the
           committed ncu summary) over that duration, against one instruction
           per scheduler per clock -- the ceiling the gathers meet first.
cpu_baseline  the CPU oracle (a restatement of the reference's PBF path, OpenMP,
           every host core) on a bounded sample of the same workload.
Multi-GPU: one single-scene replica per rank (the step does not shard without a
halo exchange), so scaling is weak.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PBF particle-steps/s (4 iters), batched vs per-scene; serving p50/p99 ms"
UNIT = "particle-steps/s"
L2_FLUSH_BYTES = 256 << 20

# Algorithmic (compulsory) bytes per particle of each kernel: every SoA array a
# kernel must touch, once; neighbour re-reads are assumed to hit in cache.
ALGO_BYTES = {
    "predict": 44,      # x, v (32) + previous key (4) -> key, index (8)
    "reorder": 112,     # key, index (8) + gather x, v, type, colour, slot (44) -> x, v, p*, type, colour, slot (60)
    "lambda": 24,       # p* (16) -> lambda, density (8)
    "delta": 36,        # p*, lambda (20) -> p* (16)
    "vorticity": 64,    # p*, v (32) -> omega, XSPH velocity (32)
    "vorticity_apply": 80,  # p*, omega, XSPH velocity (48) -> v, x (32)
}


def stage_names(iterations, baseline=True):
    names = ["predict", "sort", "reorder"]
    for _ in range(iterations):
        names += ["lambda", "delta"]
    if baseline:
        names += ["vorticity", "vorticity_apply"]
    return names


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled(kernel, workload, key="dram_bytes_per_launch"):
    """A per-launch figure of `kernel` from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", f"ncu_{kernel}_{workload}.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            return float(line.split(":", 1)[1].split()[0])
    return None


SMS, SCHEDULERS_PER_SM = 152, 4


class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_sample(seconds, params, make_scene):
    """Time the CPU oracle (all host threads) on the workload until ~`seconds` pass."""
    from oracle import oracle
    oracle.build()
    parts, cfg = make_scene()
    n = len(parts["mass"])
    steps = 0
    t0 = time.perf_counter()
    while True:
        oracle.step(params, cfg, parts)
        steps += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": f"dam_break_1m ({n} particles), the first {steps} steps from the initial state, "
                      f"{dt:.1f} s"}


# Algorithmic bytes of marching cubes: per lattice sample its value, normal and colour
# written (20); per cube its case byte, triangle count and offset (~21, the 8 corner
# values re-read from cache); per triangle its 84-byte record written.
MC_BYTES = {"sample": 20, "cube": 21, "triangle": 84}


def time_surface(batch, stream, k=0):
    """Marching cubes of scene k's current state (position grid, field, case scan,
    emit; triangles left on the device), timed with CUDA events on the solver's
    stream, with the algorithmic bytes of the lattice over that time.  The batch's
    first surface also allocates its lattice and triangle buffers (`first_ms`); `ms`
    is a second surface of the same state."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    for _ in range(2):
        batch.sync()
        e0.record(stream)
        counts = batch.surface_all()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    first_ms, ms = times
    gi = batch.grid_info(k)
    samples = int(gi.lattice[0]) * int(gi.lattice[1]) * int(gi.lattice[2])
    cubes = (int(gi.lattice[0]) - 1) * (int(gi.lattice[1]) - 1) * (int(gi.lattice[2]) - 1)
    tris = int(counts[k])
    algo = MC_BYTES["sample"] * samples + MC_BYTES["cube"] * cubes + MC_BYTES["triangle"] * tris
    peak, peak_kind = measured_peaks()
    gbs = algo / (ms * 1e-3) / 1e9
    return {"cells": [int(gi.lattice[0]) - 1, int(gi.lattice[1]) - 1, int(gi.lattice[2]) - 1], "samples": samples,
            "triangles": tris, "ms": ms, "first_ms": first_ms, "algorithmic_bytes": algo, "achieved_gbs": gbs, "hbm_frac": gbs / peak,
            "peak_kind": peak_kind, "error_flags": batch.error_flags()}


def dropin_frames(parts, cfg, warmup, frames):
    """The drop-in as a libfluid application calls it: tests/cpp/dropin_frames.cpp
    drives cuda::SphSolver::advance on a std::vector<fluid::Particle> (read and written
    in place by the library) for `warmup` + `frames` frames; returns its JSON line."""
    from libfluid_gb300 import build, capi
    lib_dir = os.path.dirname(build.build())
    exe = os.path.join(lib_dir, "dropin_frames")
    src = os.path.join(ROOT, "tests", "cpp", "dropin_frames.cpp")
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src), os.path.getmtime(build.LIB)):
        cmd = ["g++", "-std=c++14", "-O2", "-I" + os.path.join(ROOT, "include"), src, "-L" + lib_dir, "-lfluidgb",
               "-Wl,-rpath," + lib_dir, "-o", exe]
        subprocess.run(cmd, check=True, capture_output=True)
    import numpy as np
    rec = capi.to_records(parts)
    fd, path = tempfile.mkstemp(suffix=".scene")
    with os.fdopen(fd, "wb") as f:
        f.write(np.uint64(len(rec)).tobytes())
        f.write(rec.tobytes())
        f.write(np.array([cfg.dt, cfg.scale, 0.0, cfg.isolevel], np.float32).tobytes())
        f.write(np.uint32(cfg.iterations).tobytes())
        sphere = list(cfg.sphere) if cfg.sphere_enabled else [0.0, 0.0, 0.0, 0.0]
        f.write(np.array([*cfg.constant_force, *cfg.min_bound, *cfg.max_bound, *sphere], np.float32).tobytes())
    try:
        r = subprocess.run([exe, path, str(warmup), str(frames), "1"], capture_output=True, text=True, timeout=600)
    finally:
        os.unlink(path)
    if r.returncode != 0:
        return {"error": (r.stderr or "")[-300:], "rc": r.returncode}
    return json.loads(r.stdout.strip().splitlines()[-1])


def bench_batched(params, steps=100, mc_every=10, tune=True, rank=0, world=1):
    """Workload 4: 64 mixed scenes in one batch vs the same scenes stepped one by one,
    `steps` steps with every scene's surface each `mc_every`.  With several ranks
    each steps its share of the scenes (partition.local_scenes, no collective on the
    data path); an arm's time is its slowest rank's."""
    import torch
    from libfluid_gb300 import partition, scenes
    from libfluid_gb300.solver import Batch, SphSolver
    specs = scenes.batched_64()

    def run_local(mine):
        local = [spec for _, spec in mine]
        total = sum(len(p["mass"]) for p, _ in local)
        solver = SphSolver(params=params)
        if tune:
            # both arms tuned on copies: the batch's bucket, and one scene per single's bucket
            t = Batch(solver, [(scenes.copy_particles(p), c) for p, c in local])
            t.autotune(3)
            t.close()
            seen = set()
            for p, c in local:
                bucket = len(p["mass"]).bit_length()
                if bucket in seen:
                    continue
                seen.add(bucket)
                t = Batch(solver, [(scenes.copy_particles(p), c)])
                t.autotune(3)
                t.close()
        batch = Batch(solver, [(scenes.copy_particles(p), c) for p, c in local])
        batch.step(3)
        batch.sync()
        launches0 = batch.launches
        partition.barrier()
        t0 = time.perf_counter()
        tris = 0
        for s in range(1, steps + 1):
            batch.step(1)
            if s % mc_every == 0:
                tris += sum(batch.surface_all())
        batch.sync()
        t_batched = time.perf_counter() - t0
        launches = batch.launches - launches0
        batch.close()
        singles = [Batch(solver, [(scenes.copy_particles(p), c)]) for p, c in local]
        for b in singles:
            b.step(3)
        for b in singles:
            b.sync()
        partition.barrier()
        t0 = time.perf_counter()
        for s in range(1, steps + 1):
            for b in singles:
                b.step(1)
            if s % mc_every == 0:
                for b in singles:
                    b.surface_all()  # triangles left on the device, as in the batched arm
        for b in singles:
            b.sync()
        t_loop = time.perf_counter() - t0
        for b in singles:
            b.close()
        solver.close()
        # the plain single-scene step as a libfluid user calls it: one drop-in solver
        # per scene, advance() per frame with host arrays, a surface every mc_every frames
        plain = [(SphSolver(params=params), scenes.copy_particles(p), c) for p, c in local]
        for sv, p, c in plain:
            for _ in range(3):
                sv.advance(c, p)
        torch.cuda.synchronize()
        partition.barrier()
        t0 = time.perf_counter()
        for s in range(1, steps + 1):
            for sv, p, c in plain:
                c.surface = 1 if s % mc_every == 0 else 0
                sv.advance(c, p)
                c.surface = 0
        t_plain = time.perf_counter() - t0
        for sv, _, _ in plain:
            sv.close()
        torch.cuda.synchronize()
        return {"particles": total, "batched_s": t_batched, "loop_s": t_loop, "plain_s": t_plain,
                "launches": launches, "triangles": tris}

    per_rank = partition.sharded_run(specs, rank, world, run_local)
    r = partition.combine(per_rank, sum_keys=("particles", "launches", "triangles"),
                          max_keys=("batched_s", "loop_s", "plain_s"))
    total = r["particles"]
    v_b = total * steps / r["batched_s"]
    v_l = total * steps / r["loop_s"]
    v_p = total * steps / r["plain_s"]
    return {"workload": "batched_64", "scenes": len(specs), "particles": total, "steps": steps,
            "surface_every": mc_every, "ranks": world, "batched_particle_steps_per_s": v_b,
            "per_scene_loop_particle_steps_per_s": v_l, "speedup": v_b / v_l,
            "per_scene_advance_loop_particle_steps_per_s": v_p, "speedup_vs_advance_loop": v_b / v_p,
            "batched_launches": r["launches"], "triangles": r["triangles"],
            "arms": "batched: one resident batch; loop: the same scenes as resident single-scene batches; "
                    "advance loop: one drop-in solver per scene, advance() with host arrays every frame"}


def bench_large(params, steps=20, warmup=3, tune=True):
    """The 8 388 608-particle double dam break (two 128x128x256 blocks): its p* array
    (134 MB) is larger than L2, so it is the case where HBM traffic is real.  Device-
    resident steps with CUDA events on the solver stream; the whole step's algorithmic
    bytes (N x (384 + 60 I) = 624 B per particle-step at I = 4) over its duration."""
    import torch
    from libfluid_gb300 import scenes
    from libfluid_gb300.solver import Batch, SphSolver
    parts, cfg = scenes.double_dam_8m()
    n = len(parts["mass"])
    solver = SphSolver(params=params)
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    tuned = None
    if tune:
        t = Batch(solver, [(scenes.copy_particles(parts), cfg)])
        tuned = t.autotune(3)
        t.close()
    batch = Batch(solver, [(parts, cfg)])
    batch.set_timing(True)
    batch.step(warmup)
    batch.sync()
    names = stage_names(cfg.iterations)
    stage_sum = [0.0] * len(names)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total_ms = 0.0
    for _ in range(steps):
        with torch.cuda.stream(stream):
            e0.record(stream)
            batch.step(1)
            e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        for i, v in enumerate(batch.stage_times()):
            stage_sum[i] += v
    flags = batch.error_flags()
    surface = time_surface(batch, stream)  # the 512x256x256-cell lattice
    batch.close()
    solver.close()
    ms = total_ms / steps
    stages = {}
    for name, v in zip(names, stage_sum):
        stages[name] = round(stages.get(name, 0.0) + v / steps, 4)
    peak, peak_kind = measured_peaks()
    algo = n * (384 + 60 * int(cfg.iterations))
    gbs = algo / (ms * 1e-3) / 1e9
    return {"workload": "double_dam_8m", "particles": n, "steps": steps, "warmup": warmup,
            "ms_per_step": ms, "particle_steps_per_s": n / (ms * 1e-3), "stages_ms_per_step": stages,
            "step_algorithmic_bytes": algo, "step_achieved_gbs": gbs, "hbm_peak_gbs": peak,
            "hbm_peak_kind": peak_kind, "step_hbm_frac": gbs / peak, "error_flags": flags, "surface": surface,
            "autotuned": ({"block": int(tuned.block), "skin_h": round(float(tuned.skin), 3),
                           "persistent": bool(tuned.persistent),
                           "particles_per_thread": int(tuned.particles_per_thread),
                           "verlet_lists": bool(tuned.verlet)} if tuned else None)}


def bench_ref_profile(steps=30, warmup=5, tune=True):
    """The 1M dam break under the reference's own constants (the profile the C++
    drop-in uses by default: no XSPH or vorticity, colour diffusion instead), device-
    resident steps timed with CUDA events on the solver stream."""
    import torch
    from libfluid_gb300 import capi, scenes
    from libfluid_gb300.solver import Batch, SphSolver
    params = capi.params(capi.PROFILE_REF, 0.1)
    parts, cfg = scenes.dam_break_1m()
    n = len(parts["mass"])
    solver = SphSolver(params=params)
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    if tune:
        t = Batch(solver, [(scenes.copy_particles(parts), cfg)])
        t.autotune(3)
        t.close()
    batch = Batch(solver, [(parts, cfg)])
    batch.step(warmup)
    batch.sync()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    total = 0.0
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            batch.step(1)
            e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    flags = batch.error_flags()
    batch.close()
    solver.close()
    ms = total / steps
    return {"workload": "dam_break_1m", "profile": "ref", "particles": n, "steps": steps, "warmup": warmup,
            "ms_per_step": ms, "particle_steps_per_s": n / (ms * 1e-3), "error_flags": flags}


def bench_serving(params, requests=48, run_seconds=25.0, seed=5, tick_particles=0, log_path=None, rank=0, world=1):
    """Workload 5: saturation throughput, then a Poisson stream at 80% of it.  With
    several ranks every rank draws the same streams and serves the requests a
    replicated Router gives it (partition.route_stream): the job's throughput is the
    ranks' particle-steps over the slowest rank's time, latencies are pooled."""
    import numpy as np
    from libfluid_gb300 import partition, scenes
    from libfluid_gb300.serve import Server
    from libfluid_gb300.solver import SphSolver
    cache = {}

    def scene_for(n):
        if n not in cache:
            cache[n] = scenes.cube_scene(n, 5000 + len(cache))
        return cache[n]

    stream = scenes.serving_stream(requests, 1.0, seed=seed)
    work = [(n, st, mesh) for _, n, st, mesh, _ in stream]
    mean_ps = float(np.mean([n * st for n, st, _ in work]))
    mine = [w for _, w in partition.route_stream(work, rank, world, n_of=lambda w: w[0], steps_of=lambda w: w[1])]
    solver = SphSolver(params=params)

    def saturate(one_at_a_time):
        sv = Server(solver, one_at_a_time=one_at_a_time, tick_particles=tick_particles)
        partition.barrier()
        tickets = []
        for n, st, mesh in mine:
            p, c = scene_for(n)
            tickets.append(sv.submit(c, p, st, mesh))
        sv.drain(1200)
        s = sv.stats()
        for t in tickets:
            sv.fetch(t)
        sv.close()
        return s

    s_sat = saturate(False)
    s_loop = saturate(True)
    sat_all = partition.gather_summary((s_sat.particle_steps, s_sat.elapsed_seconds, s_loop.particle_steps,
                                        s_loop.elapsed_seconds))
    sat = sum(x[0] for x in sat_all) / max(x[1] for x in sat_all)
    loop = sum(x[2] for x in sat_all) / max(x[3] for x in sat_all)
    rate = 0.8 * sat / mean_ps
    arrivals = scenes.serving_stream(100000, rate, seed=seed + 1)
    arrivals = [a for a in arrivals if a[0] <= run_seconds]
    mine_arr = [a for _, a in partition.route_stream(arrivals, rank, world)]
    sv = Server(solver, tick_particles=tick_particles)
    partition.barrier()
    t0 = time.perf_counter()
    tickets = []
    for t_arr, n, st, mesh, _ in mine_arr:
        delay = t_arr - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        p, c = scene_for(n)
        tickets.append(sv.submit(c, p, st, mesh))
    sv.drain(1200)
    res = [sv.poll(t) for t in tickets]
    lat = sv.step_latencies()
    tick_scenes = sv.tick_scenes()
    tick_parts = sv.tick_particles()
    tick_starts = sv.tick_starts()
    tick_steps = sv.tick_steps()
    s = sv.stats()
    for t in tickets:
        sv.fetch(t)
    sv.close()
    solver.close()
    req = np.array([r.t_done - r.t_submit for r in res if r.status == 2])
    if log_path and rank == 0:
        np.savez(log_path, latency=lat, scenes=tick_scenes, particles=tick_parts, starts=tick_starts,
                 steps=tick_steps, request_latency=req)
    # the latency each request saw for its next state: every request of a tick waits
    # that tick's time (a tick of k steps hands over k steps at once)
    per_req = np.repeat(lat, tick_scenes[:len(lat)]) if len(tick_scenes) >= len(lat) else lat
    # time per request-step: a tick's time over the steps it advanced
    per_step = np.repeat(lat / np.maximum(tick_steps[:len(lat)], 1), tick_scenes[:len(lat)])
    pooled = partition.gather_summary({"lat": lat, "req": req, "per_req": per_req, "per_step": per_step,
                                       "ticks_steps": tick_steps, "requests": len(tickets),
                                       "completed": int(s.completed), "particle_steps": s.particle_steps,
                                       "elapsed": s.elapsed_seconds, "rebuilds": int(s.rebuilds),
                                       "rebuild_s": s.rebuild_seconds, "sat_rebuilds": int(s_sat.rebuilds)})
    lat = np.concatenate([p["lat"] for p in pooled])
    req = np.concatenate([p["req"] for p in pooled])
    per_req = np.concatenate([p["per_req"] for p in pooled])
    per_step = np.concatenate([p["per_step"] for p in pooled])
    ks = np.concatenate([p["ticks_steps"] for p in pooled])
    pct = lambda a, q: float(np.percentile(a, q)) * 1e3 if len(a) else None  # noqa: E731
    return {"workload": "serving", "ranks": world, "saturation_particle_steps_per_s": sat,
            "one_at_a_time_particle_steps_per_s": loop, "batching_gain": sat / loop,
            "offered_fraction_of_saturation": 0.8, "arrival_rate_per_s": rate,
            "requests": sum(p["requests"] for p in pooled), "completed": sum(p["completed"] for p in pooled),
            "particle_steps_per_s": sum(p["particle_steps"] for p in pooled) / max(p["elapsed"] for p in pooled),
            "step_ms": {"p50": pct(lat, 50), "p95": pct(lat, 95), "p99": pct(lat, 99)},
            "request_ms": {"p50": pct(req, 50), "p95": pct(req, 95), "p99": pct(req, 99)},
            "p99_over_p50_step": (pct(lat, 99) / pct(lat, 50)) if len(lat) else None,
            "request_step_ms": {"p50": pct(per_req, 50), "p95": pct(per_req, 95), "p99": pct(per_req, 99)},
            "p99_over_p50_request_step": (pct(per_req, 99) / pct(per_req, 50)) if len(per_req) else None,
            "steps_per_tick": {"mean": float(ks.mean()) if len(ks) else None,
                               "max": int(ks.max()) if len(ks) else None,
                               "multi_step_fraction": float((ks > 1).mean()) if len(ks) else None},
            "per_step_ms": {"p50": pct(per_step, 50), "p95": pct(per_step, 95), "p99": pct(per_step, 99)},
            "latency_note": "step_ms: tick latency, the time a request waits for its next state (a tick "
                            "advances its group by one step, or by several when the group holds less than "
                            "half the tick budget); per_step_ms: that time over the steps the tick advanced",
            "rebuilds": sum(p["rebuilds"] for p in pooled), "rebuild_s": sum(p["rebuild_s"] for p in pooled),
            "saturation_rebuilds": sum(p["sat_rebuilds"] for p in pooled)}


REF_ARM_BUDGET_S = 150.0  # wall time the reference arm's timed steps may take


def run_reference(args):
    """The reference's own CPU implementation of the path, on the host cores: its
    OpenMP solver cpu::SphSolver (include/fluid/cpusph.hpp:75-240), compiled from the
    reference's source with two patches (return type, return statement) over a
    project-written GLM subset (oracle/patch_cpusph.py, oracle/cpusph_driver.cpp).
    One step is one advance() of the whole dam_break_1m scene, as a libfluid
    application calls it; the timed steps stop early when they would run past
    REF_ARM_BUDGET_S.  Where the solver could not be built, the oracle port (a
    restatement of the same path) is timed instead and the line says so."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from libfluid_gb300 import capi, scenes
    from oracle import oracle
    oracle.build()
    parts, cfg = scenes.dam_break_1m()
    n = len(parts["mass"])
    if oracle.RefCpuSolver.available():
        solver = oracle.RefCpuSolver(0.1, parts)
        cores = solver.threads()
        for _ in range(args.warmup):
            solver.advance(cfg, 1)
        times = []
        for _ in range(args.steps):
            times.append(solver.advance(cfg, 1))
            if sum(times) + times[-1] > REF_ARM_BUDGET_S:
                break
        solver.close()
        kind = "reference"
        note = ("the reference's cpu::SphSolver (include/fluid/cpusph.hpp) with its own constants (rho0 6378, "
                "CFM 600, damping 0.49; no XSPH, vorticity or collider), k-d tree neighbours within 2h, "
                "OpenMP on every host core")
    else:
        params = capi.default_params(capi.PROFILE_BASELINE, 0.1)
        cores = oracle.num_threads()
        for _ in range(args.warmup):
            oracle.step(params, cfg, parts)
        times = []
        for _ in range(args.steps):
            t = time.perf_counter()
            oracle.step(params, cfg, parts)
            times.append(time.perf_counter() - t)
        kind = "port"
        note = ("the reference's CPU solver was not built (its patched sources were absent); this arm times the "
                "CPU oracle, a restatement of the path")
    done = len(times)
    total = sum(times)
    value = n * done / total
    sample = f"dam_break_1m ({n} particles), advance() steps {args.warmup + 1}..{args.warmup + done}"
    if done < args.steps:
        sample += f" ({done} of the {args.steps} asked, stopped at the {REF_ARM_BUDGET_S:.0f} s budget)"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * total / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        # the same keys as our arm's config; the reference's CPU solver has no sphere
        # collider and no L2 to flush
        "config": {"workload": "dam_break_1m", "particles": n, "iterations": 4, "sphere_collider": False,
                   "l2": "not applicable (CPU)", "parallelism": f"cpu x{cores} threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": note,
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from libfluid_gb300 import build, capi, scenes
    from libfluid_gb300.solver import Batch, SphSolver
    build.build()
    params = capi.params(capi.PROFILE_BASELINE, 0.1)
    parts, cfg = scenes.dam_break_1m()
    parts0 = scenes.copy_particles(parts)  # the initial state, for the full-run and drop-in legs
    n = len(parts["mass"])
    solver = SphSolver(params=params)
    # a dedicated (non-legacy) stream: the library launches its graphs on it and the
    # CUDA events below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    solver.set_stream(stream.cuda_stream)
    # autotune on a copy of the scene (so the timed steps stay steps 5-55 of the
    # dam break); the solver caches the launch shape for this size bucket
    tuner = Batch(solver, [(scenes.copy_particles(parts), cfg)])
    tuned = tuner.autotune(3) if not args.no_tune else None
    tuner.close()
    batch = Batch(solver, [(parts, cfg)])
    direct_io = batch.host_io_direct()
    batch.set_timing(True)
    for _ in range(args.warmup):
        batch.step(1)
    batch.sync()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    names = stage_names(cfg.iterations)
    stage_sum = [0.0] * len(names)
    clocks = Clocks(local)
    launches0 = batch.launches
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    step_ms = []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        flush.zero_()
        ev0.record(stream)
        batch.step(1)
        ev1.record(stream)
        ev1.synchronize()
        step_ms.append(ev0.elapsed_time(ev1))
        st = batch.stage_times()
        for i, t in enumerate(st[:len(names)]):
            stage_sum[i] += t
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    launches = batch.launches - launches0
    flags = batch.error_flags()
    total_s = sum(step_ms) / 1e3
    t = torch.tensor([total_s], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_s = float(t.item())
    value = n * args.steps * world / max_s

    # roofline of the dominant kernel
    per_kernel = {}
    for nm, tot in zip(names, stage_sum):
        k = per_kernel.setdefault(nm, [0.0, 0])
        k[0] += tot
        k[1] += 1
    gathers = {k: v for k, v in per_kernel.items() if k in ALGO_BYTES}
    dom = max(gathers, key=lambda k: gathers[k][0])
    launches_dom = gathers[dom][1] * args.steps
    mean_ms = gathers[dom][0] / launches_dom
    algo = ALGO_BYTES[dom] * n
    achieved = algo / (mean_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    # the summary's figures for the configuration the autotuner chose (near rows with
    # or without Verlet lists)
    with_lists = tuned is None or bool(tuned.verlet)
    suffix = "_with_lists" if with_lists else ""
    traffic = profiled(dom, "dam_break_1m", "dram_bytes_per_launch" + suffix)
    # the FP32-issue ceiling of the same kernel: its warp instructions per launch
    # (ncu) over the live launch time, against one instruction per scheduler per clock
    inst = profiled(dom, "dam_break_1m", "warp_inst_per_launch" + suffix)
    issue = None
    if inst:
        mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
        ipeak = SMS * SCHEDULERS_PER_SM * mhz * 1e6
        iach = inst / (mean_ms / 1e3)
        issue = {"bound": "fp32-issue", "achieved": iach, "peak": ipeak, "unit": "warp-inst/s",
                 "frac": iach / ipeak, "warp_inst_per_launch": inst, "sm_mhz": mhz}
    step_total = sum(stage_sum) / args.steps

    # end to end through the reference-facing call with host buffers
    # the same window of the dam break as the device-resident measurement: W frames
    # of warm-up, then K timed frames
    e2e_steps = args.steps
    host = scenes.copy_particles(parts)
    e2e_solver = SphSolver(params=params)
    if tuned is not None:
        t = Batch(e2e_solver, [(scenes.copy_particles(parts), cfg)])
        t.autotune(3)
        t.close()
    for _ in range(args.warmup):
        e2e_solver.advance(cfg, host)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_solver.advance(cfg, host)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = n * e2e_steps * world / float(te.item())
    e2e_solver.close()

    # the 200-step run of the workload as stated, from the initial state: every step
    # device-resident (no L2 flush: one continuous run), then the end-of-run surface
    # of the 256x128x128-cell lattice; and the same 200 frames through fgb_advance
    full_run = None
    if world == 1 and not args.no_extra:
        full_steps = 200
        fb = Batch(solver, [(scenes.copy_particles(parts0), cfg)])
        fb.sync()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        fb.step(full_steps)
        f1.record(stream)
        f1.synchronize()
        dev_ms = f0.elapsed_time(f1) / full_steps
        surface = time_surface(fb, stream)
        ff = fb.error_flags()
        fb.close()
        host_full = scenes.copy_particles(parts0)
        fs = SphSolver(params=params)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(full_steps):
            fs.advance(cfg, host_full)
        e2e_full_s = time.perf_counter() - t0
        fs.close()
        full_run = {"steps": full_steps, "device_ms_per_step": dev_ms,
                    "device_particle_steps_per_s": n / (dev_ms * 1e-3),
                    "e2e_ms_per_frame": 1e3 * e2e_full_s / full_steps,
                    "e2e_particle_steps_per_s": n * full_steps / e2e_full_s, "error_flags": ff,
                    "surface_end_of_run": surface}

    # the drop-in as an application calls it: cuda::SphSolver::advance on a
    # std::vector<fluid::Particle>, the same window as e2e (W frames, then K timed)
    dropin = None
    if rank == 0 and world == 1 and not args.no_extra:
        d = dropin_frames(parts0, cfg, args.warmup, args.steps)
        if "ms_per_frame" in d:
            dropin = {"value": n / (d["ms_per_frame"] * 1e-3), "unit": UNIT, "ms_per_frame": d["ms_per_frame"],
                      "frames": d["frames"], "call": "cuda::SphSolver::advance (C++, std::vector<fluid::Particle>)",
                      "vs_e2e": (n / (d["ms_per_frame"] * 1e-3)) / e2e_value}
        else:
            dropin = d

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_sample(args.cpu_seconds, params, scenes.dam_break_1m)
    batched = serving = large = ref_profile = None
    if not args.no_extra:
        # the scene-sharded legs run on every rank (each its share); the single-scene
        # legs on one GPU
        batched = bench_batched(params, tune=not args.no_tune, rank=rank, world=world)
        if world == 1:
            large = bench_large(params, tune=not args.no_tune)
            ref_profile = bench_ref_profile(tune=not args.no_tune)
        serving = bench_serving(params, log_path=args.serving_log, rank=rank, world=world)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": max_s * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "dam_break_1m", "particles": n, "iterations": int(cfg.iterations),
                       "sphere_collider": True, "l2": "flushed (256 MiB write) before every timed step",
                       "parallelism": f"replicas x{world}"},
            "setup": {"cuda_graph": True,
                      "autotuned": ({"block": int(tuned.block), "skin_h": round(float(tuned.skin), 3),
                                     "persistent": bool(tuned.persistent),
                                     "particles_per_thread": int(tuned.particles_per_thread),
                                     "verlet_lists": bool(tuned.verlet),
                                     "trial_steps": int(tuned.steps)} if tuned else None)},
            # direct: kernels read id/type/mass/colour/position/velocity (44 B) from the
            # caller's arrays and write them back; staged: pinned float4 x, float4 v,
            # type, colour up (40 B), the same plus the upload slot down (44 B)
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": (44 if direct_io else 40) * n,
                    "d2h_bytes_per_step": 44 * n, "steps": e2e_steps, "call": "fgb_advance",
                    "host_io": "direct" if direct_io else "staged"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes_per_launch": algo,
                         "mean_launch_ms": mean_ms, "issue": issue},
            "stages_ms_per_step": {nm: round(v[0] / args.steps, 4) for nm, v in per_kernel.items()},
            "stage_sum_ms_per_step": step_total,
            "cpu_baseline": cpu,
            "e2e_dropin": dropin,
            "full_run": full_run,
            "clocks": clk,
            "gpu_launches": launches,
            "error_flags": flags,
            "batched": batched,
            "serving": serving,
            "large": large,
            "ref_profile": ref_profile,
        }
        print(json.dumps(line), flush=True)
    batch.close()
    solver.close()
    if dist:
        dist.destroy_process_group()


def ncu_case(profile="baseline", deep=0):
    """Four plain steps of dam_break_1m (per step: predict, 2 + passes sort kernels,
    reorder, list build, 4 x (lambda, delta), 2 vorticity kernels in the baseline
    profile; colour diffusion instead in the ref profile), then one surface of the
    256x128x128-cube lattice (position keys, sort, gather, field, scan, emit); with
    deep > 0, `deep` steps before those four (a flow that has broken)."""
    from libfluid_gb300 import build, capi, scenes
    from libfluid_gb300.solver import Batch, SphSolver
    build.build()
    params = capi.params(capi.PROFILE_REF if profile == "ref" else capi.PROFILE_BASELINE, 0.1)
    parts, cfg = scenes.dam_break_1m()
    solver = SphSolver(params=params)
    batch = Batch(solver, [(parts, cfg)])
    if deep:
        batch.step(deep)
    batch.step(4)
    batch.sync()
    tris = batch.surface(0)
    print("ncu case done, error flags", batch.error_flags(), "triangles", len(tris))
    batch.close()
    solver.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and serving legs")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (default launch shapes)")
    ap.add_argument("--serving-log", default=None,
                    help="write the serving leg's tick log (latency, scenes, particles, start) to this .npz")
    ap.add_argument("--ncu-deep", type=int, default=0, help="steps of --ncu-case before its four")
    ap.add_argument("--ncu-case", action="store_true",
                    help="run 4 untimed steps of the workload and exit (the case that ncu captures)")
    ap.add_argument("--ncu-profile", default="baseline", choices=["baseline", "ref"],
                    help="physics profile of --ncu-case")
    args = ap.parse_args()
    if args.ncu_case:
        ncu_case(args.ncu_profile, args.ncu_deep)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
