"""Benchmark of the GB300 FDTD engine on the single-large-job workload.

Workload (L256): 256^3 cells (257^3 = 16.97 M nodes) on a uniform 0.5 mm
mesh, 8-cell UPML on all six faces, 40 seeded dielectric bricks, a 50 ohm
z-directed lumped port with a Gaussian pulse; FP32 fields.  One bench step
is one full 1000-timestep simulation of that job (the hot path
Engine::IterateTS over the whole grid, 1000 times), with the engine's
fields reset to zero before each step.  Inputs (fields + operator, > 500 MB)
are larger than the 129 MB L2, so no explicit flush is done.

    value   Mcell-updates/s (node count x timesteps / device time, the
            reference's own MC/s convention, openems.cpp:1303-1305), device
            time = CUDA events on the engine stream around each step
    e2e     the same metric through the C ABI with host buffers: per step,
            fdtd_engine_create_compressed from the pinned compressed operator
            (host -> device), fdtd_engine_iterate over all timesteps (the
            probe / energy samples collect in the device ring), the sample
            record read back (device -> host), fdtd_engine_destroy
    roofline  the dominant half-step kernel against the measured HBM copy
            bandwidth (MEASURED_PEAKS.json)
    cpu_baseline  the oracle's restated SSE-compressed multithreaded engine
            (the reference's default engine family) on the host cores, on
            the oracle's own operator build; a table of L256 (all cores and
            one), P64 and a D192 window
    batch / serve  the B96 persistent batch against job-by-job and
            concurrent plain engines, and the serving stream against one job
            at a time (jobs/s, p50 / p99 latency, Mcell-updates/s)

--impl reference times that CPU engine alone on the same workload and metric.
Multi-GPU (torchrun): every rank runs an independent replica of the job
(the path has no exchange step: "replicas only"), value is the sum over
ranks divided by the slowest rank's time.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

TIMESTEPS = 1000
BYTES_BASE_HALF = 38      # 3 V + 3 I read, 3 V (or I) written, 2 B index
BYTES_UPML_HALF = 24      # 3 flux read + 3 flux written


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_from_profiles(kernel: str):
    """DRAM bytes per launch of the kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "ncu_traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 3 and parts[0] == kernel and parts[1] == "l256":
            try:
                return float(parts[2])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(threads: int = 0):
    from wipems_gb300 import CompressedOperator, Operator, scenes
    t0 = time.perf_counter()
    sc = scenes.l256(nr_ts=TIMESTEPS)
    op = Operator(sc, threads=threads)
    t1 = time.perf_counter()
    cop = CompressedOperator(op)
    t2 = time.perf_counter()
    return sc, op, cop, dict(operator_build_s=round(t1 - t0, 3), compress_s=round(t2 - t1, 3))


WORKLOAD = ("L256: 256^3 cells (257^3 nodes), 0.5 mm uniform mesh, UPML-8 on 6 faces, 40 seeded dielectric "
            "bricks, 50 ohm z lumped port, Gaussian f0=fc=10 GHz; one step = one "
            f"{TIMESTEPS}-timestep simulation")


def config_dict(num_lines, extra=None):
    """The workload keys both arms report (the same for the engine and the
    reference arm)."""
    n = num_lines
    d = {"workload": WORKLOAD, "nodes": n[0] * n[1] * n[2], "cells": (n[0] - 1) * (n[1] - 1) * (n[2] - 1),
         "timesteps_per_step": TIMESTEPS, "l2_policy": "inputs larger than L2 (fields+operator > 500 MB)",
         "parallelism": "replicas"}
    if extra:
        d.update(extra)
    return d


def oracle_operator(name: str, threads: int):
    """A workload's operator built by the oracle from the recorded scene,
    without the engine library (for the CPU legs)."""
    import oracle
    from wipems_gb300 import scenes
    with scenes.spec_only():
        sc = {"l256": lambda: scenes.l256(nr_ts=TIMESTEPS), "p64": lambda: scenes.p64(),
              "d192": lambda: scenes.d192()}[name]()
    return oracle.Operator(sc.spec, threads=threads)


def _oracle_rate(op, threads: int, target_s: float, max_steps: int):
    """Mcell-updates/s of the oracle's SSE-compressed x-slab engine on about
    target_s of stepping (at most max_steps timesteps)."""
    import oracle
    r = oracle.run(op.desc, [], 2, 0, engine=oracle.SSE_COMPRESSED_MT, threads=threads, energy=False, fields=False)
    per = max(r["seconds"] / 2, 1e-4)
    n = int(max(4, min(max_steps, target_s / per)))
    r = oracle.run(op.desc, [], n, 0, engine=oracle.SSE_COMPRESSED_MT, threads=threads, energy=False, fields=False)
    nodes = op.num_lines[0] * op.num_lines[1] * op.num_lines[2]
    return nodes * n / r["seconds"] / 1e6, n, r["seconds"]


def cpu_baseline(threads: int):
    """The CPU table: the oracle's restated SSE-compressed multithreaded
    engine (the reference's default engine family) on its own operator
    build, on all host cores and on one, for L256 (bounded samples), P64
    (the full 2000 timesteps) and a 300-timestep window of D192."""
    import platform
    out = {}
    l256 = oracle_operator("l256", threads)
    v, n, sec = _oracle_rate(l256, threads, 12.0, 400)
    out["l256"] = {"value": round(v, 2), "timesteps": n, "seconds": round(sec, 2), "threads": threads}
    v1, n1, sec1 = _oracle_rate(l256, 1, 8.0, 100)
    out["l256_1thread"] = {"value": round(v1, 2), "timesteps": n1, "seconds": round(sec1, 2), "threads": 1}
    del l256
    p64 = oracle_operator("p64", threads)
    for key, th in (("p64", threads), ("p64_1thread", 1)):
        vv, nn, ss = _oracle_rate(p64, th, 1e9, 2000)
        out[key] = {"value": round(vv, 2), "timesteps": nn, "seconds": round(ss, 2), "threads": th}
    del p64
    d192 = oracle_operator("d192", threads)
    vv, nn, ss = _oracle_rate(d192, threads, 1e9, 300)
    out["d192_window"] = {"value": round(vv, 2), "timesteps": nn, "seconds": round(ss, 2), "threads": threads}
    del d192
    cpu = platform.processor() or platform.machine()
    try:
        out_l = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out_l.splitlines():
            if ln.lower().startswith("model name"):
                cpu = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"value": round(v, 2), "unit": "Mcell-updates/s", "cores": threads, "kind": "port",
            "sample": f"{n} timesteps of L256 ({sec:.1f} s) with the restated SSE-compressed x-slab "
                      f"multithreaded engine on the oracle's own operator build",
            "nproc": os.cpu_count(), "cpu": cpu, "machine": platform.machine(), "table": out}


def batch_and_serve(args, device: int) -> dict:
    """D192 on the plain engine (the graded / dispersive configuration, with
    its voltage kernel's algorithmic bandwidth), and the two patterns beside
    the plain engine, measured on this GPU:
    batch -- the 96-job B96 sweep (1500 timesteps each) as one persistent
    batch against the plain engine job by job and against the same engines
    run concurrently on their own streams (CUDA events / wall clock);
    serve -- a seeded Poisson stream of serving requests (operator builds
    included) through the continuous-batching server against the same
    stream one job at a time through the plain engine (wall clock from the
    first submission), with p50 / p99 job latency."""
    from wipems_gb300 import workloads
    out = {}
    d = workloads.single("d192", device=device)
    peak, _ = _peaks()
    out["d192"] = {
        "workload": "D192: 192^3 cells (193^3 nodes) on a seeded graded mesh (0.2-1 mm), UPML-8, Drude (~25 %) and "
                    "Lorentz (~15 %) bricks; 3000 timesteps, factorized geometry",
        "mcells": round(d["mcells"], 1), "device_ms": round(d["device_ms"], 2), "tiling": d["tiling"],
        "tuples_e": d["tuples_e"], "tuples_h": d["tuples_h"],
        "ms_volt": round(d["ms_volt"], 5), "ms_curr": round(d["ms_curr"], 5),
        "volt_algorithmic_bytes": d["volt_algorithmic_bytes"], "volt_gbs": round(d["volt_gbs"], 1),
        "volt_frac": round(d["volt_gbs"] / peak, 4),
        "timing": "CUDA events; kernel times from 20 single launches each"}
    b = workloads.b96(96, 1500, device)
    out["batch"] = {
        "workload": "B96: 96 seeded jobs, grid edges 48-160 cells per axis, half PEC / half UPML-8, 1-10 "
                    "dielectric bricks, one 50 ohm port, f0 in 1-20 GHz; 1500 timesteps each",
        "jobs": b["jobs"], "nodes": b["nodes"], "timesteps": b["timesteps"],
        "batched_mcells": round(b["batched_mcells"], 1), "job_by_job_mcells": round(b["plain_mcells"], 1),
        "concurrent_mcells": round(b["concurrent_mcells"], 1),
        "ratio_vs_job_by_job": round(b["speedup"], 3),
        "ratio_vs_concurrent": round(b["batched_mcells"] / b["concurrent_mcells"], 3),
        "batched_ms": round(b["batched_ms"], 2), "job_by_job_ms": round(b["plain_ms"], 2),
        "concurrent_wall_s": round(b["concurrent_wall_s"], 3), "tiling": b["tiling"],
        "timing": "batched and job by job: CUDA events; concurrent: wall clock"}
    sv = workloads.serve(n_jobs=args.serve_jobs, mean_gap=args.serve_gap, device=device)
    S, P = sv["served"], sv["plain"]
    keep = ("wall_s", "jobs_per_s", "mcells", "p50_s", "p99_s", "gpu_ms", "gpu_mcells")
    out["serve"] = {
        "workload": f"S: {args.serve_jobs} seeded Poisson requests (mean gap {args.serve_gap * 1e3:.0f} ms), grid "
                    "edges log-uniform 32-256 cells, 60 % dielectric + UPML-8, 40 % Drude or Lorentz; each job "
                    "stops at -40 dB energy or 20000 timesteps; operator builds included",
        "jobs": sv["jobs"], "served": {k: round(S[k], 4) for k in keep},
        "one_at_a_time": {k: round(P[k], 4) for k in keep},
        "ratio": round(sv["speedup"], 3), "gpu_ratio": round(sv["gpu_speedup"], 3),
        "same_stop_timesteps": sv["same_stop_timesteps"], "failed": S["failed"],
        "timing": "wall clock over the stream (first submission to last completion); latency = completion "
                  "minus arrival"}
    return out


def max_over_ranks(vals, device):
    """The slowest rank's figures: elementwise max over all ranks of a list
    of floats (unchanged with one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in vals]
    t = torch.tensor([float(v) for v in vals], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def run_reference(args, rank, world):
    """The reference's CPU algorithm (the oracle's restated SSE-compressed
    x-slab multithreaded engine) on the oracle's own operator build of the
    same L256 scene: neither the scene, nor the operator, nor the stepping
    touches the engine library."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle
    op = oracle_operator("l256", threads)
    nodes = op.num_lines[0] * op.num_lines[1] * op.num_lines[2]
    per_step = max(4, args.ref_timesteps)
    for _ in range(args.warmup):
        oracle.run(op.desc, [], per_step, 0, engine=oracle.SSE_COMPRESSED_MT, threads=threads, energy=False,
                   fields=False)
    tot = 0.0
    for _ in range(args.steps):
        r = oracle.run(op.desc, [], per_step, 0, engine=oracle.SSE_COMPRESSED_MT, threads=threads, energy=False,
                       fields=False)
        tot += r["seconds"]
    value = nodes * per_step * args.steps / tot / 1e6
    line = {"metric": "Mcell-updates/s", "value": round(value, 2), "unit": "Mcell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": config_dict(op.num_lines),
            "cpu_baseline": {"value": round(value, 2), "unit": "Mcell-updates/s", "cores": threads, "kind": "port",
                             "sample": f"{per_step} timesteps of L256 per step (restated SSE-compressed "
                                       f"x-slab multithreaded engine on the oracle's operator build); the rate "
                                       f"is per timestep, so the step count does not change it"},
            "e2e": {"value": round(value, 2), "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, local_rank):
    import torch
    import wipems_gb300
    from wipems_gb300 import Engine
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
    sc, op, cop, setup = build_workload()
    nodes = op.num_nodes
    # kernel tiling from the project's autotuner (setup, not timed)
    from wipems_gb300 import autotune
    t_tune = time.perf_counter()
    best, _ = autotune.tune(cop, stages=(3, 4), xchunks=(4, 8, 16), steps=100, device=local_rank)
    setup["autotune_s"] = round(time.perf_counter() - t_tune, 2)
    tiling = dict(stages=best["stages"], x_chunk=best["x_chunk"], kernel=best["kernel"], tile_y=best["tile_y"])
    eng = Engine(cop, device=local_rank, max_timesteps=TIMESTEPS, **tiling)
    setup["tiling"] = {"stages": best["stages"], "x_chunk": best["x_chunk"], "tile_y": eng.stats()["tile_y"],
                       "tile": f"32z x {eng.stats()['tile_y']}y", "kernel": best["kernel"],
                       "searched": "tile_y 4/8, stages 3/4, x_chunk 4/8/16 (CUDA events, graph chunks)"}
    # warm-up
    for _ in range(args.warmup):
        eng.reset()
        eng.iterate(TIMESTEPS)
    launches = 0
    ms_total = 0.0
    sampler = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.reset()
        eng.iterate(TIMESTEPS)
        ms, n = eng.last_timing()
        ms_total += ms
        launches += n
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    if dist:
        dist.barrier()
    dev_s = ms_total / 1e3
    dev_s, wall = max_over_ranks([dev_s, wall], "cuda")
    value = nodes * TIMESTEPS * args.steps * world / dev_s / 1e6

    # live per-kernel durations (events around each launch)
    eng.reset()
    ms_v, ms_c = eng.profile_kernels(60)
    upml = cop.info["num_upml_nodes"]
    bytes_half = BYTES_BASE_HALF * nodes + BYTES_UPML_HALF * upml
    if tiling["kernel"] == "fused":  # one kernel per timestep: the whole step's algorithmic bytes
        dominant, ms_dom, bytes_launch = "k_step_fused", ms_v, 2 * bytes_half
    else:
        dominant, ms_dom = ("k_volt", ms_v) if ms_v >= ms_c else ("k_curr", ms_c)
        bytes_launch = bytes_half
    peak, peak_kind = _peaks()
    achieved = bytes_launch / (ms_dom / 1e3) / 1e9
    traffic = _traffic_from_profiles(dominant)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": dominant,
                "algorithmic_bytes_per_launch": bytes_launch, "launch_ms": round(ms_dom, 5),
                "other_kernel_ms": round(ms_c if dominant == "k_volt" else ms_v, 5),
                "step_frac": round(2 * bytes_half / ((ms_v + ms_c) / 1e3) / 1e9 / peak, 4),
                "peak_kind": f"{peak_kind} (HBM copy, MEASURED_PEAKS.json)" if peak_kind == "measured" else peak_kind}
    eng.close()

    # e2e through the C ABI with host buffers, as many simulations as the device leg
    e2e_steps = max(1, args.steps)
    h2d = cop.info["host_bytes"]
    d2h = 0
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(e2e_steps):
        # one simulation through the API: upload the compressed operator,
        # run all timesteps (the samples stay in the device ring), read the
        # probe / energy record back
        e = Engine(cop, device=local_rank, max_timesteps=TIMESTEPS, **tiling)
        e.iterate(TIMESTEPS)
        n = e.num_samples()
        ts, vals, en = e.read_samples(0, n)
        d2h += ts.nbytes + vals.nbytes + en.nbytes + 4
        e.close()
    torch.cuda.synchronize()
    te = time.perf_counter() - te
    e2e_value = nodes * TIMESTEPS * e2e_steps * world / te / 1e6

    extra = {}
    if rank == 0 and args.extras:
        extra = batch_and_serve(args, local_rank)
    if rank == 0:
        threads = os.cpu_count() or 1
        cpu = cpu_baseline(threads)
        line = {"metric": "Mcell-updates/s", "value": round(value, 2), "unit": "Mcell-updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_s / args.steps * 1e3, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config_dict(op.num_lines),
                "engine": {**setup, "wall_s": round(wall, 3), "upml_nodes": cop.info["num_upml_nodes"],
                           "tuples_e": cop.info["num_tuples_e"], "tuples_h": cop.info["num_tuples_h"],
                           "index_bytes": cop.info["index_bytes_e"]},
                "roofline": roofline,
                "cpu_baseline": cpu,
                "e2e": {"value": round(e2e_value, 2), "unit": "Mcell-updates/s",
                        "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h // e2e_steps),
                        "steps": e2e_steps},
                "gpu_launches": int(launches), "clocks": clocks, **extra}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-timesteps", type=int, default=20, help="CPU timesteps per reference-arm step")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the batch (B96) and serving-stream measurements")
    ap.add_argument("--serve-jobs", type=int, default=200, help="requests in the serving stream")
    ap.add_argument("--serve-gap", type=float, default=0.02, help="mean Poisson gap between requests (s)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend=backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            import __graft_entry__
            __graft_entry__.build()
            run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
