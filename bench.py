"""Benchmark of the GB300 particle-mesh engine on the README workload.

Workload (one "step" = one PM step of the hot path): 256^3 particles on a 512^3 grid,
box 250 Mpc/h, LCDM (Om 0.3, OL 0.7, h 0.7, ns 0.96, reference normalisation), seeded
GRF + Zel'dovich ICs at a = 0.02, leapfrog with da = 0.98/1000 (1000 STEPS).  The timed
steps are the first K steps of that run.

  value   resident engine (pm_batch_*): state in HBM, K steps timed with CUDA events
          (graph replays), particle-updates/s = 256^3 * K / time.
  e2e     the drop-in loop through the C ABI on HOST arrays (pm_step_host): every step
          copies positions+velocities in from pinned host memory and back out.
  roofline  the phase with the largest share of the step, from CUDA events recorded on
          the launch stream around each phase (pm_batch_profile), against its
          algorithmic bytes.
  cpu_baseline  the CPU port of the reference step (oracle/: C + OpenMP particle loops,
          scipy.fft) on all host cores, one bounded sample of full-size steps.

``--impl reference`` times only that CPU port (the reference itself needs numba and
pyFFTW, which are not installed) and prints its own line.  With torchrun and N > 1 each
rank runs an independent replica ("replicas only": one simulation does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cosmological-particle-mesh-simulation_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "particle-updates/s (plain vs batched/served) at P(k)≤0.5% err; p50/p99 sim latency"
UNIT = "particle-updates/s"
WORKLOAD = ("README workload: 256^3 particles, 512^3 grid, box 250 Mpc/h, LCDM, seeded GRF + "
            "Zel'dovich ICs at a=0.02, 1000 leapfrog steps to a=1 (first K steps timed)")
FALLBACK_HBM_GBS = 6800.0


def workload_config(steps_needed: int, n_parts=256, n_cells=512, box=250.0):
    from pmgpu.config import Config, step_count
    cfg = Config(n_parts=n_parts, n_cells=n_cells, box_size=box, random_seed=0, steps=1000, power=0.96,
                 omega_m0=0.3, omega_b0=0.04, omega_k0=0.0, omega_lambda0=0.7, h0=0.7, a_init=0.02, a_end=1.0)
    if step_count(cfg.a_init, cfg.a_end, cfg.steps) < steps_needed:
        # keep da, extend the end so that the driver loop runs at least steps_needed steps
        cfg.a_end = cfg.a_init + (steps_needed + 2) * cfg.da
        cfg.steps = steps_needed + 2
    return cfg


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def max_over_ranks(x, dist=None, device="cpu"):
    """The maximum of a per-rank float over all ranks: the slowest replica bounds the job."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def job_throughput(particles, steps, ranks, seconds):
    """Whole-job particle-updates/s: every rank advances its own replica by `steps` steps."""
    return particles * steps * ranks / seconds


def host_link(local, nbytes, reps=5):
    """Host-link bandwidth between pinned host memory and this GPU (GB/s): one direction at a
    time, and both at once on two streams (the copies the e2e step makes each step)."""
    import torch
    n = nbytes // 4
    h_in = torch.empty(n, dtype=torch.float32).pin_memory()
    h_out = torch.empty(n, dtype=torch.float32).pin_memory()
    d_a = torch.empty(n, dtype=torch.float32, device=f"cuda:{local}")
    d_b = torch.empty(n, dtype=torch.float32, device=f"cuda:{local}")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def run(h2d, d2h):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            if h2d:
                with torch.cuda.stream(s1):
                    d_a.copy_(h_in, non_blocking=True)
            if d2h:
                with torch.cuda.stream(s2):
                    h_out.copy_(d_b, non_blocking=True)
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps

    run(True, True)  # warm-up
    t_in, t_out, t_both = run(True, False), run(False, True), run(True, True)
    return {"h2d": round(nbytes / t_in / 1e9, 1), "d2h": round(nbytes / t_out / 1e9, 1),
            "both_each_way": round(nbytes / t_both / 1e9, 1), "bytes": nbytes}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profiled_traffic():
    """Per-launch DRAM bytes (dram__bytes_read.sum + write.sum) of each phase's kernel from
    the committed ncu summary, scaled to the full workload there; None if absent."""
    path = os.path.join(ROOT, "profiles", "resident_step_256p_512g_launches.md")
    out = {}
    try:
        for line in open(path):
            if line.startswith("traffic:"):
                _, k, v = line.split()
                out[k] = float(v)
    except OSError:
        pass
    return out


def algorithmic_bytes(np_, n):
    """Bytes each phase must move once (inputs read once, outputs written once)."""
    nc = n ** 3
    h = n * n * (n // 2 + 1)
    return {
        # the resident step fuses the deposit with the x R2C: particles in, spectrum rows out
        "deposit": 12 * np_ + 8 * h,
        "x_r2c": 0,
        "y_fwd": 16 * h,
        "z_green": 16 * h,
        "y_inv": 16 * h,
        "x_c2r": 8 * h + 4 * nc,
        "kick": 24 * np_ + 4 * nc + 24 * np_,
        "sort": 0, "rows": 0, "coef": 0,
    }


def bench_config(cfg, ws, t_ics):
    """The `config` object of both arms' lines (same keys, same workload description)."""
    return {"workload": WORKLOAD if (cfg.n_parts, cfg.n_cells) == (256, 512) else
            f"reduced case: {cfg.n_parts}^3 particles, {cfg.n_cells}^3 grid",
            "n_parts": cfg.n_parts, "n_cells": cfg.n_cells, "box_size": cfg.box_size, "a_init": cfg.a_init,
            "da": cfg.da, "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "l2": f"inputs larger than L2 ({cfg.n_cells}^3 grid = {4 * cfg.n_cells ** 3 / 1e6:.0f} MB per field)",
            "ics_seconds": round(t_ics, 1)}


def make_ics(cfg):
    from pmgpu import ics
    return ics.initial_conditions(cfg)


def run_gpu(args, ws, rank, local):
    import numpy as np
    import torch

    import pmgpu
    from pmgpu.batch import Batch
    from pmgpu.context import PMContext

    torch.cuda.set_device(local)
    pmgpu.build()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))

    def barrier():
        if dist is not None:
            dist.barrier()

    K, W = args.steps, args.warmup
    cfg = workload_config(max(K, W + args.profile_steps), args.n_parts, args.n_cells, args.box)
    t0 = time.time()
    pos, vel = make_ics(cfg)
    t_ics = time.time() - t0
    np_ = cfg.np_total

    # ---- warm-up on a throwaway batch (W steps, graphs instantiated), then a per-phase
    # CUDA-event profile of the next steps of that run ----------------------------------
    wb = Batch(device=local, autotune=not args.no_autotune)
    wb.add(cfg, pos, vel)
    wb.step(max(W, 1))
    prof = wb.profile(args.profile_steps)
    wb.check_device()
    wb.close()
    del wb

    # ---- timed: K steps of a fresh run from the ICs --------------------------------
    b = Batch(device=local, autotune=not args.no_autotune)
    sid = b.add(cfg, pos, vel)
    b.step(0)
    launches = b.launches_per_step()
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk, torch.cuda.stream(stream):
        ev0.record(stream)
        b.step(K)  # enqueued on `stream` (graph replays)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    b.check_device()
    _, done = b.state(sid)
    if done != K:
        raise RuntimeError(f"ran {done} steps instead of {K}")
    b.close()

    t_max = max_over_ranks(ms, dist, "cuda")
    value = job_throughput(np_, K, ws, t_max / 1e3)

    # ---- e2e: drop-in loop on host arrays through the C ABI -------------------------
    e2e = None
    if args.e2e_steps > 0:
        ctx = PMContext(cfg, device=local)
        hp = torch.from_numpy(pos.copy()).pin_memory()
        hv = torch.from_numpy(vel.copy()).pin_memory()
        a = cfg.a_init
        ctx.step_host(hp, hv, cfg.mass, a, cfg.da)  # warm-up (allocations)
        hp.copy_(torch.from_numpy(pos))
        hv.copy_(torch.from_numpy(vel))
        torch.cuda.synchronize()
        barrier()
        te0 = time.perf_counter()
        for i in range(args.e2e_steps):
            ctx.step_host(hp, hv, cfg.mass, a, cfg.da)
            a += cfg.da
        torch.cuda.synchronize()
        te = time.perf_counter() - te0
        ctx.check_device()
        te = max_over_ranks(te, dist, "cuda")
        e2e = {"value": job_throughput(np_, args.e2e_steps, ws, te), "unit": UNIT,
               "h2d_bytes_per_step": 2 * 3 * 4 * np_, "d2h_bytes_per_step": 2 * 3 * 4 * np_,
               "steps": args.e2e_steps, "api": "pm_step_host (C ABI, pinned host arrays)"}
        ctx.close()
        # the host link the step's copies cross: its floor is the step's bytes each way at the
        # bandwidth both directions reach together
        link = host_link(local, 2 * 3 * 4 * np_)
        e2e["host_link_gbs"] = link
        e2e["link_floor_ms"] = round(2 * 3 * 4 * np_ / (link["both_each_way"] * 1e9) * 1e3, 3)
        e2e["ms_per_step"] = round(te / args.e2e_steps * 1e3, 3)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant phase --------------------------------------------
    alg = algorithmic_bytes(np_, cfg.n_cells)
    dom = max((k for k in prof if alg.get(k, 0) > 0), key=lambda k: prof[k])
    peak, peak_src = measured_peak()
    achieved = alg[dom] / (prof[dom] / 1e3) / 1e9
    traffic = profiled_traffic().get(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_src,
                "traffic": traffic, "algorithmic_bytes": alg[dom], "launch_ms": round(prof[dom], 4),
                "phase_ms": {k: round(v, 4) for k, v in prof.items()},
                # every phase with algorithmic bytes: achieved / measured peak
                "phase_frac": {k: round(alg[k] / (prof[k] / 1e3) / 1e9 / peak, 4) for k in prof
                               if alg.get(k, 0) > 0 and prof[k] > 0},
                "step_ms_sum_of_phases": round(sum(prof.values()), 4)}

    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(cfg, pos, vel, args.cpu_steps)
    # the other two workloads of the metric, on the same GPU (single-GPU runs only)
    batched = served = None
    if ws == 1 and not args.plain_only:
        batched = measure_batched(args, local)
        served = measure_served(args, local, args.headline_serve_seconds)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": t_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: seeded GRF + Zel'dovich ICs (reference algorithm)",
        "config": bench_config(cfg, ws, t_ics),
        "e2e": e2e, "gpu_launches": launches * K, "roofline": roofline, "cpu_baseline": cpu,
        "clocks": clk.summary(), "batched": batched, "served": served,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def cpu_baseline(cfg, pos, vel, steps):
    """The reference step on all host cores: the C + OpenMP restatement of its particle
    loops (oracle/cpu_step.c, float64 arithmetic on the float32 state, threads over
    particles like the reference's numba prange) and scipy.fft for the Poisson solve."""
    import numpy as np
    cores = len(os.sched_getaffinity(0))
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    from oracle import cpu_port as C
    from oracle import pm_oracle as O
    C.load()
    fg = O.fourier_grid(cfg.n_cells)
    p, v = np.array(pos, dtype=np.float32), np.array(vel, dtype=np.float32)
    a = cfg.a_init
    t0 = time.perf_counter()
    for _ in range(steps):
        C.step(p, v, cfg.mass, a, cfg.da, cfg, fg, workers=cores)
        a += cfg.da
    t = time.perf_counter() - t0
    return {"value": cfg.np_total * steps / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} full-size step(s) ({cfg.n_parts}^3 particles, {cfg.n_cells}^3 grid) of the CPU port "
                      f"of the reference step: particle loops in C + OpenMP on {cores} threads, FFTs in scipy.fft "
                      f"(complex128) on {cores} threads",
            "seconds": round(t, 2)}


def _ics_pool(cfgs, workers=16):
    import concurrent.futures as cf
    import multiprocessing as mp
    from pmgpu import ics
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(ics.initial_conditions, cfgs))


def batched_configs(count=64, seed=0):
    """Ensemble of independent simulations: seeds 0..count-1, N_PARTS uniform in {32, 48, 64,
    96, 128}, grid 2 N_PARTS, box uniform in [50, 500] Mpc/h, 200 steps each."""
    import numpy as np
    from pmgpu.config import Config
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(rng.choice([32, 48, 64, 96, 128]))
        out.append(Config(n_parts=n, n_cells=2 * n, box_size=float(rng.uniform(50.0, 500.0)), random_seed=s,
                          steps=200))
    return out


def batched_ics(cfgs, device):
    """Initial conditions of every configuration, generated on the GPU (host draws only the
    uniform pairs of the reference's rejection loop)."""
    from pmgpu.device_ics import DeviceICs
    gens, out = {}, []
    for c in cfgs:
        g = gens.get(c.n_parts) or gens.setdefault(c.n_parts, DeviceICs(c.n_parts, device))
        out.append(g.generate(c))
    for g in gens.values():
        g.close()
    return out


def measure_batched(args, local):
    """All simulations of the ensemble in one batch (one launch per phase, CUDA graphs)
    against each one run alone, one after another: dict of the figures."""
    import torch
    from pmgpu.batch import Batch
    from pmgpu.config import step_count
    cfgs = batched_configs(args.batch_sims)
    t0 = time.time()
    ics_ = batched_ics(cfgs, local)
    t_ics = time.time() - t0
    steps = [step_count(c.a_init, c.a_end, c.steps) for c in cfgs]
    pu = sum(c.np_total * k for c, k in zip(cfgs, steps))
    # warm-up on the same ensemble: graphs instantiated, and the launch schedule of each grid
    # size tuned (once per process, like an FFT planner) before anything is timed
    warm = Batch(device=local)
    for c, (p, v) in zip(cfgs, ics_):
        warm.add(c, p, v)
    warm.step(4)  # (a plan is tuned once it has run two steps)
    schedule = warm.schedule()
    warm.close()
    for c, (p, v) in zip(cfgs, ics_):  # and each simulation alone, for the comparison run
        one = Batch(device=local)
        one.add(c, p, v)
        one.step(3)
        one.close()
    stream = torch.cuda.Stream()

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    def wall(fn):  # host seconds of set-up work, the device idle on both sides
        torch.cuda.synchronize()
        t = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t

    b, setup_batch = wall(lambda: Batch(device=local))
    ids, t_add = wall(lambda: [b.add(c, p, v) for c, (p, v) in zip(cfgs, ics_)])
    setup_batch += t_add
    t_batch = timed(lambda: b.step(max(steps) + 1))
    b.check_device()
    assert all(b.state(i)[1] == k for i, k in zip(ids, steps))
    b.close()
    pb = Batch(device=local)
    for c, (p, v) in zip(cfgs, ics_):
        pb.add(c, p, v)
    pb.step(2)
    prof = pb.profile(3)
    launches = pb.launches_per_step()
    pb.close()

    # each simulation alone: its set-up (batch, admission) on the host clock, its steps on the
    # device clock, like the batched run's
    t_plain, setup_plain, by_size = 0.0, 0.0, {}
    for c, (p, v) in zip(cfgs, ics_):
        one, t_new = wall(lambda: Batch(device=local))
        _, t_one_add = wall(lambda: one.add(c, p, v))
        t_one = timed(lambda: one.step(step_count(c.a_init, c.a_end, c.steps) + 1))
        one.close()
        t_plain += t_one
        setup_plain += t_new + t_one_add
        by_size[c.n_cells] = by_size.get(c.n_cells, 0.0) + t_one
    return {"value": pu / t_batch, "unit": UNIT, "plain_value": pu / t_plain,
            "batched_over_plain": t_plain / t_batch,
            "batched_over_plain_with_setup": (t_plain + setup_plain) / (t_batch + setup_batch),
            "sims": len(cfgs), "particle_updates": pu,
            "seconds_batched": round(t_batch, 3), "seconds_plain": round(t_plain, 3),
            "setup_seconds_batched": round(setup_batch, 3), "setup_seconds_plain": round(setup_plain, 3),
            "seconds_plain_by_grid": {k: round(v, 3) for k, v in sorted(by_size.items())},
            "ics_seconds": round(t_ics, 2),
            "batched_phase_ms": {k: round(v, 4) for k, v in prof.items()}, "launches_per_step": launches,
            "schedule": schedule,
            "workload": f"{len(cfgs)} simulations, seeds 0-{len(cfgs) - 1}, N_PARTS in {{32,48,64,96,128}}, "
                        "grid 2N, box U(50,500) Mpc/h, 200 steps, f32",
            "plain": "each simulation alone in its own resident batch, one after another"}


def measure_served(args, local, seconds):
    """Poisson request stream against one GPU (continuous batching under a memory cap)."""
    from pmgpu.serve import Server, poisson_stream, summarize
    stream = poisson_stream(args.serve_rate, seconds, seed=0)
    srv = Server(mem_cap_bytes=int(args.serve_cap_gb * 2 ** 30), ic_workers=args.ic_workers,
                 steps_per_tick=args.steps_per_tick, device=local)
    t0 = time.perf_counter()
    res = srv.run(stream)
    wall = time.perf_counter() - t0
    host = srv.host_seconds()
    srv.close()
    summ = summarize(res, wall)
    offered = sum(r.particle_updates for r in stream) / seconds
    return {"value": summ["particle_updates_per_s"], "unit": UNIT, "p50_latency_s": summ["p50_latency_s"],
            "p99_latency_s": summ["p99_latency_s"], "mean_latency_s": summ["mean_latency_s"],
            "requests": summ["requests"], "offered_requests": len(stream),
            "offered_particle_updates_per_s": offered, "wall_s": round(wall, 2), "host_seconds": host,
            "workload": f"Poisson {args.serve_rate} req/s for {seconds} s, N_PARTS in {{64,96,128,192,256}} weighted "
                        "40/25/20/10/5%, grid 2N, box U(100,500), steps U(50,500), f32",
            "memory_cap_gb": args.serve_cap_gb, "steps_per_tick": args.steps_per_tick}


def run_batched(args, local):
    import pmgpu
    import torch
    torch.cuda.set_device(local)
    pmgpu.build()
    d = measure_batched(args, local)
    line = {"metric": METRIC, "workload": "batched", **d, "dtype": "f32",
            "data": "synthetic: seeded GRF + Zel'dovich ICs (reference algorithm)"}
    print(json.dumps(line), flush=True)


def run_served(args, local):
    import pmgpu
    import torch
    torch.cuda.set_device(local)
    pmgpu.build()
    with ClockSampler(local) as clk:
        d = measure_served(args, local, args.serve_seconds)
    line = {"metric": METRIC, "workload": "served", **d, "dtype": "f32", "data": "synthetic request stream (seeded)",
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_gradient(args, local):
    """The force of the step two ways on the same state: the reference's central differences of
    phi (32 taps per particle) and the spectral gradient (three force grids, 8 taps per axis),
    each as pm_step on device arrays (K steps after W, CUDA events)."""
    import dataclasses
    import pmgpu
    import torch
    from pmgpu.context import PMContext
    torch.cuda.set_device(local)
    pmgpu.build()
    cfg = workload_config(args.steps + args.warmup, args.n_parts, args.n_cells, args.box)
    pos, vel = make_ics(cfg)
    res = {}
    for name, c in (("central_difference", cfg), ("spectral_gradient", dataclasses.replace(cfg, spectral_gradient=True))):
        ctx = PMContext(c, device=local)
        p, v = torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda()
        a = cfg.a_init
        for _ in range(args.warmup):
            ctx.step(p, v, cfg.mass, a, cfg.da)
            a += cfg.da
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            ctx.step(p, v, cfg.mass, a, cfg.da)
            a += cfg.da
        e1.record()
        torch.cuda.synchronize()
        ctx.check_device()
        ms = e0.elapsed_time(e1) / args.steps
        res[name] = {"ms_per_step": round(ms, 4), "value": cfg.np_total / (ms / 1e3)}
        ctx.close()
    line = {"metric": METRIC, "workload": "gradient", "unit": UNIT, "steps": args.steps, "warmup": args.warmup,
            **res, "config": bench_config(cfg, 1, 0.0), "api": "pm_step on device arrays (drop-in step)"}
    print(json.dumps(line), flush=True)


def run_sizes(args, local):
    """Per grid size: a batch of one size, particles on a grid twice as fine and the README
    workload's resolution (box 250 N_PARTS / 256 Mpc/h), about 16.8M particles in all; the CUDA
    event time of each phase of a step after --warmup steps (default 20 here), and its
    achieved GB/s on the phase's algorithmic bytes."""
    import pmgpu
    import torch
    from pmgpu.batch import Batch
    from pmgpu.config import Config
    from pmgpu.device_ics import DeviceICs
    torch.cuda.set_device(local)
    pmgpu.build()
    peak, _ = measured_peak()
    rows = []
    for npart, count in ((32, 96), (48, 64), (64, 48), (96, 19), (128, 8), (192, 3), (256, 1)):
        gen = DeviceICs(npart, local)
        b = Batch(device=local)
        for s in range(count):
            c = Config(n_parts=npart, n_cells=2 * npart, box_size=250.0 * npart / 256, random_seed=s, steps=1000)
            p, v = gen.generate(c)
            b.add(c, p, v)
        gen.close()
        b.step(max(args.warmup, 20))
        prof = b.profile(5)
        b.check_device()
        n, np_ = 2 * npart, count * npart ** 3
        alg = {k: v * count for k, v in algorithmic_bytes(npart ** 3, n).items()}  # per simulation, times count
        phases = {k: {"ms": round(v, 4), **({"gbs": round(alg[k] / (v / 1e3) / 1e9),
                                              "frac": round(alg[k] / (v / 1e3) / 1e9 / peak, 3)}
                                             if alg.get(k, 0) > 0 and v > 0 else {})}
                  for k, v in prof.items() if v > 0.003}
        rows.append({"n_cells": n, "sims": count, "particles": np_, "step_ms": round(sum(prof.values()), 4),
                     "ns_per_particle": round(sum(prof.values()) * 1e6 / np_, 4), "phases": phases,
                     "schedule": b.schedule()[0]})
        b.close()
    print(json.dumps({"metric": METRIC, "workload": "sizes", "unit": "ms per phase", "peak_gbs": peak,
                      "rows": rows}), flush=True)


def run_reference(args, ws, rank):
    """The reference's step on the host cores (its CPU port, see cpu_baseline): W untimed
    full-size steps, then the K timed steps the command asks for, on the same workload and
    with the same config keys as the GPU arm."""
    if rank != 0:
        return
    K, W = max(1, args.steps), max(0, args.warmup)
    cfg = workload_config(K + W, args.n_parts, args.n_cells, args.box)
    t0 = time.time()
    pos, vel = make_ics(cfg)
    t_ics = time.time() - t0
    if W > 0:
        cpu_baseline(cfg, pos, vel, W)
    cb = cpu_baseline(cfg, pos, vel, K)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": ws, "steps": K,
            "warmup": W, "ms_per_step": cb["seconds"] * 1e3 / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded GRF + Zel'dovich ICs (reference algorithm)",
            "config": bench_config(cfg, ws, t_ics),
            "note": "numba/pyFFTW are not installed: the reference step runs as its CPU port (C + OpenMP "
                    "particle loops, scipy.fft complex128 FFTs, all host cores), full-size steps",
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=999)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--profile-steps", type=int, default=5)
    # full-size CPU steps timed (about 1.7 s each on 16 Arm cores: a 10 s sample)
    ap.add_argument("--cpu-steps", type=int, default=6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-parts", type=int, default=256, help="reduced cases for profiling only")
    ap.add_argument("--n-cells", type=int, default=512)
    ap.add_argument("--box", type=float, default=250.0)
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "served", "gradient", "sizes"],
                    help="plain: the README workload (headline); batched / served: the ensemble and "
                         "request-stream workloads")
    ap.add_argument("--batch-sims", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-seconds", type=float, default=120.0,
                    help="arrival window of --workload served (the stream's specified 120 s)")
    ap.add_argument("--headline-serve-seconds", type=float, default=20.0,
                    help="arrival window of the served figures carried by the default (plain) line")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the batch engine's default launch schedule (fixed launch order, for profiling)")
    ap.add_argument("--plain-only", action="store_true",
                    help="the plain line without its batched and served figures")
    ap.add_argument("--serve-cap-gb", type=float, default=150.0)
    ap.add_argument("--steps-per-tick", type=int, default=4)
    ap.add_argument("--ic-workers", type=int, default=12)
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload == "batched":
        if rank == 0:
            run_batched(args, local)
    elif args.workload == "served":
        if rank == 0:
            run_served(args, local)
    elif args.workload == "gradient":
        if rank == 0:
            run_gradient(args, local)
    elif args.workload == "sizes":
        if rank == 0:
            run_sizes(args, local)
    else:
        run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    main()
