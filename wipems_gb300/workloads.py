"""Measurement drivers for the workloads beside the L256 headline of
bench.py: the P64 and D192 single jobs, the B96 batched sweep and the S
serving stream.  Each prints one JSON object.

    python -m wipems_gb300.workloads p64|d192|b96|serve [options]

Timings are CUDA-event device times unless named wall (host clock around a
whole stream, including operator builds).  Mcell-updates/s uses the node
count (lines product), the reference's convention (openems.cpp:1303-1305).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def single(kind: str, steps: int = 0, device: int = 0) -> dict:
    """One job on the plain engine (CUDA graphs, TMA kernels, autotuned)."""
    from . import CompressedOperator, Engine, Operator, autotune, scenes
    sc = {"p64": scenes.p64, "d192": scenes.d192}[kind]()
    t0 = time.perf_counter()
    op = Operator(sc)
    cop = CompressedOperator(op)
    setup = time.perf_counter() - t0
    best, _ = autotune.tune(cop, stages=(3, 4), steps=40, device=device)
    nts = steps or sc.nr_ts
    eng = Engine(cop, device=device, max_timesteps=nts + 100, stages=best["stages"], x_chunk=best["x_chunk"],
                 kernel=best["kernel"], tile_y=best["tile_y"])
    eng.iterate(min(nts, 50))     # warm-up (graph instantiation)
    eng.reset()
    eng.iterate(nts)
    ms, launches = eng.last_timing()
    mv, mc = eng.profile_kernels(20)
    n = op.num_nodes
    info = cop.info
    ade_e = lor_e = 0
    if info["num_ade_nodes"]:  # voltage-side Lorentz/Drude nodes and the Lorentz ones among them (flag words)
        fe = cop.expand()[4]
        ade_e = int(np.count_nonzero(fe & 2))
        lor_e = int(np.count_nonzero(fe & 4))
    # algorithmic bytes of one voltage launch: 38 B per node, 24 B per UPML
    # node (flux read + write), 24 B per Lorentz/Drude state read + write
    volt_bytes = 38 * n + 24 * info["num_upml_nodes"] + 24 * ade_e + 24 * lor_e
    return dict(workload=kind, nodes=n, timesteps=nts, device_ms=ms, mcells=n * nts / (ms / 1e3) / 1e6,
                kernel=best["kernel"],
                ms_volt=mv, ms_curr=mc, launches=launches, setup_s=round(setup, 3), tiling=best,
                tuples_e=info["num_tuples_e"], tuples_h=info["num_tuples_h"],
                geometry_factored=info["geometry_factored"], upml_nodes=info["num_upml_nodes"],
                ade_nodes=info["num_ade_nodes"], ade_volt_nodes=ade_e, lorentz_volt_nodes=lor_e,
                volt_algorithmic_bytes=volt_bytes, volt_gbs=volt_bytes / (mv / 1e3) / 1e9)


def extensions(steps: int = 1000, device: int = 0) -> list:
    """The cost of the extensions around the hot path on the L256 grid
    (256^3 cells, 40 bricks, 50 ohm port), one tiling for all variants:
    UPML-8 (the headline), PEC walls, Mur on all faces, UPML-8 with 64
    frequency-domain probe frequencies, UPML-8 with four lumped RLC
    elements (two series, two parallel) beside the port."""
    from . import CompressedOperator, Engine, Operator, autotune, scenes
    from .fdtd import BC_MUR, BC_PEC

    def variant(name):
        sc = scenes.l256(nr_ts=steps)
        if name == "pec":
            sc.set_boundary([BC_PEC] * 6, [0] * 6)
        elif name == "mur":
            sc.set_boundary([BC_MUR] * 6, [0] * 6)
        elif name == "rlc":
            L = scenes.uniform_lines(256, 0.5)
            c = 128
            for k, series in enumerate((True, True, False, False)):
                x = L[c - 6 + 4 * k]
                sc.add_lumped_rlc([x, L[c + 5], L[c - 2]], [x, L[c + 5], L[c + 2]], 2, R=25.0 + 10 * k,
                                  L=2e-9, Cap=0.5e-12, series=series, caps=False, priority=900)
        return sc

    out = []
    best = None
    for name in ("upml", "pec", "mur", "fd", "rlc"):
        op = Operator(variant(name))
        cop = CompressedOperator(op)
        if best is None:
            best, _ = autotune.tune(cop, stages=(3, 4), steps=40, device=device)
        eng = Engine(cop, device=device, max_timesteps=steps + 100, stages=best["stages"], x_chunk=best["x_chunk"],
                     kernel=best["kernel"], tile_y=best["tile_y"])
        if name == "fd":
            eng.set_frequencies(np.linspace(1e9, 20e9, 64))
        eng.iterate(50)  # warm-up (graph instantiation)
        eng.reset()
        eng.iterate(steps)
        ms, launches = eng.last_timing()
        n = op.num_nodes
        out.append(dict(workload="l256_" + name, nodes=n, timesteps=steps, device_ms=round(ms, 3),
                        mcells=round(n * steps / (ms / 1e3) / 1e6, 1), launches=launches,
                        us_per_step=round(ms * 1e3 / steps, 2), tiling=best))
        del eng, cop, op
    base = out[0]["us_per_step"]
    for r in out:
        r["vs_upml"] = round(r["us_per_step"] / base, 4)
    return out


def b96(n_jobs: int = 96, timesteps: int = 1500, device: int = 0) -> dict:
    """B96: the seeded 96-job sweep, plain engine job by job vs one batch
    (autotuned x_chunk / graph length)."""
    from . import Batch, CompressedOperator, Engine, Operator, autotune, scenes
    t0 = time.perf_counter()
    cops, nodes = [], []
    for s in range(n_jobs):
        op = Operator(scenes.b96_job(s, nr_ts=timesteps))
        cops.append(CompressedOperator(op))
        nodes.append(op.num_nodes)
    setup = time.perf_counter() - t0
    work = sum(nodes) * timesteps
    plain_ms = 0.0
    for c in cops:
        e = Engine(c, device=device, max_timesteps=timesteps)
        e.iterate(timesteps)
        plain_ms += e.last_timing()[0]
        e.close()
    best, table = autotune.tune_batch(cops, device=device)
    engines = [Engine(c, device=device, max_timesteps=timesteps, kernel="tma") for c in cops]
    b = Batch(engines, x_chunk=best["x_chunk"], graph_steps=best["graph_steps"], blocks_per_sm=best["blocks_per_sm"],
              chains=best.get("chains", 1), tile_y=best.get("tile_y", 8))
    b.iterate(timesteps)
    st = b.stats()
    b.close()
    for e in engines:
        e.close()
    # the same jobs as concurrent plain engines (one stream each)
    engines = [Engine(c, device=device, max_timesteps=timesteps) for c in cops]
    for e in engines:
        e.iterate(0)  # uploads done, first sample taken
    t0 = time.perf_counter()
    for e in engines:
        e.iterate_async(timesteps)
    for e in engines:
        e.wait()
    conc_s = time.perf_counter() - t0
    for e in engines:
        e.close()
    plain = work / (plain_ms / 1e3) / 1e6
    batched = work / (st["last_ms"] / 1e3) / 1e6
    return dict(workload="b96", jobs=n_jobs, timesteps=timesteps, nodes=sum(nodes), setup_s=round(setup, 2),
                plain_ms=plain_ms, plain_mcells=plain, batched_ms=st["last_ms"], batched_mcells=batched,
                speedup=batched / plain, concurrent_wall_s=conc_s, concurrent_mcells=work / conc_s / 1e6,
                tiling=best, groups=st["num_groups"], work_items=st["work_items"],
                persistent_blocks=st["persistent_blocks"], launches=st["last_launches"])


def serve(n_jobs: int = 48, mean_gap: float = 0.02, end_crit: float = 1e-4, seed: int = 777, device: int = 0,
          round_steps: int = 128, modes=("served", "plain"), batch_min_jobs: int = 0,
          build_workers: int = 0, tile_share: int = 0, max_active: int = 0) -> dict:
    """S: a seeded Poisson stream of serve_job requests (operator build
    included), through the continuous-batching server and one at a time
    through the plain engine.  Both stop every job at -40 dB energy or its
    NrTS; the stopping timesteps are compared."""
    from . import CompressedOperator, Engine, Operator, Server, scenes
    rng = np.random.default_rng(seed)
    arr = np.cumsum(rng.exponential(mean_gap, n_jobs))
    arr -= arr[0]
    out = dict(workload="serve", jobs=n_jobs, mean_gap_s=mean_gap, end_crit=end_crit, seed=seed,
               round_steps=round_steps, batch_min_jobs=batch_min_jobs, tile_share=tile_share, max_active=max_active)

    def pct(a, q):
        return float(np.percentile(np.asarray(a), q))

    ts_served = ts_plain = None
    if "served" in modes:
        srv = Server(device=device, round_steps=round_steps, batch_min_jobs=batch_min_jobs,
                     build_workers=build_workers, tile_share=tile_share, max_active=max_active)
        t0 = time.perf_counter()
        ids = []
        for k in range(n_jobs):
            dt = arr[k] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(scenes.serve_job(k), end_crit=end_crit))
        srv.wait(0)
        st = [srv.status(i) for i in ids]
        ss = srv.stats()
        srv.close()
        lat = [x["t_done"] - x["t_submit"] for x in st]
        mk = max(x["t_done"] for x in st) - min(x["t_submit"] for x in st)
        work = sum(x["nodes"] * x["timesteps"] for x in st)
        ts_served = [x["timesteps"] for x in st]
        out["served"] = dict(wall_s=mk, mcells=work / mk / 1e6, jobs_per_s=n_jobs / mk, p50_s=pct(lat, 50),
                             p99_s=pct(lat, 99), gpu_ms=ss["gpu_ms"], gpu_mcells=work / (ss["gpu_ms"] / 1e3) / 1e6,
                             rounds=ss["rounds"], rebuilds=ss["rebuilds"], peak_gb=ss["peak_bytes"] / 1e9,
                             failed=ss["jobs_failed"], node_steps=work)
    if "plain" in modes:
        t0 = time.perf_counter()
        lat, ts_plain, work, gpu_ms = [], [], 0, 0.0
        for k in range(n_jobs):
            dt = arr[k] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            sc = scenes.serve_job(k)
            op = Operator(sc)
            e = Engine(CompressedOperator(op), device=device, end_crit=end_crit)
            while not e.done and e.num_timesteps < sc.nr_ts:
                e.iterate(min(1024, sc.nr_ts - e.num_timesteps))
                gpu_ms += e.last_timing()[0]
            e.samples()
            ts_plain.append(e.num_timesteps)
            work += op.num_nodes * e.num_timesteps
            e.close()
            lat.append(time.perf_counter() - t0 - arr[k])
        mk = time.perf_counter() - t0
        out["plain"] = dict(wall_s=mk, mcells=work / mk / 1e6, jobs_per_s=n_jobs / mk, p50_s=pct(lat, 50),
                            p99_s=pct(lat, 99), gpu_ms=gpu_ms, gpu_mcells=work / (gpu_ms / 1e3) / 1e6,
                            node_steps=work)
    if ts_served is not None and ts_plain is not None:
        out["same_stop_timesteps"] = ts_served == ts_plain
        out["speedup"] = out["served"]["mcells"] / out["plain"]["mcells"]
        out["gpu_speedup"] = out["served"]["gpu_mcells"] / out["plain"]["gpu_mcells"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["p64", "d192", "b96", "serve", "ext"])
    ap.add_argument("--jobs", type=int, default=0)
    ap.add_argument("--timesteps", type=int, default=0)
    ap.add_argument("--gap", type=float, default=0.02)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--batch-min", type=int, default=0,
                    help="serve: run the persistent batch with at least this many resident jobs (0 = never)")
    ap.add_argument("--served-only", action="store_true")
    ap.add_argument("--workers", type=int, default=0, help="serve: host build workers (0 = the server's default)")
    ap.add_argument("--round-steps", type=int, default=128, help="serve: timesteps per scheduling round")
    ap.add_argument("--max-active", type=int, default=0, help="serve: cap on resident jobs (0 = the server's default)")
    ap.add_argument("--tile-share", type=int, default=0,
                    help="serve: tile each job for 1/N of the SMs (0 = the server's default, 1 = the job alone)")
    args = ap.parse_args()
    if args.workload in ("p64", "d192"):
        r = single(args.workload, args.timesteps, args.device)
    elif args.workload == "b96":
        r = b96(args.jobs or 96, args.timesteps or 1500, args.device)
    elif args.workload == "ext":
        r = extensions(args.timesteps or 1000, args.device)
    else:
        r = serve(args.jobs or 48, args.gap, device=args.device, batch_min_jobs=args.batch_min,
                  build_workers=args.workers, tile_share=args.tile_share, round_steps=args.round_steps,
                  max_active=args.max_active,
                  modes=("served",) if args.served_only else ("served", "plain"))
    print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
