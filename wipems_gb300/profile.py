"""Profiling driver: builds one workload and runs a few timesteps, so that an
external profiler (ncu) can capture the half-step kernels.

    python -m wipems_gb300.profile --workload l256|p64|d192|l160|b96|l256mur --steps 8 [--graphs]
        [--tile-y 4|8] [--x-chunk N] [--blocks-per-sm B --chains C (b96)]

Kernels are launched individually (no CUDA graph) unless --graphs is given,
so a launch list shows every E / H kernel separately.
"""
from __future__ import annotations

import argparse
import time


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="l256", choices=["l256", "p64", "d192", "l160", "b96", "l256mur"])
    ap.add_argument("--jobs", type=int, default=24, help="b96: number of sweep jobs (seeds 0..jobs-1)")
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--graphs", action="store_true")
    ap.add_argument("--tile-y", type=int, default=0)
    ap.add_argument("--x-chunk", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0, help="b96: batch schedule (-1 = one block per item)")
    ap.add_argument("--chains", type=int, default=0, help="b96: job-range chains per kernel variant")
    args = ap.parse_args()
    from . import Batch, CompressedOperator, Engine, Operator, scenes
    if args.workload == "b96":  # batched mode, one step per launch sequence (no graph)
        t0 = time.perf_counter()
        cops = [CompressedOperator(Operator(scenes.b96_job(s))) for s in range(args.jobs)]
        engines = [Engine(c, kernel="tma") for c in cops]
        b = Batch(engines, x_chunk=args.x_chunk, graph_steps=1, blocks_per_sm=args.blocks_per_sm, chains=args.chains,
                  tile_y=args.tile_y)
        t1 = time.perf_counter()
        b.iterate(args.steps)
        st = b.stats()
        n = st["total_nodes"]
        print(f"b96[{args.jobs}]: nodes={n} setup={t1 - t0:.2f}s steps={args.steps} device_ms={st['last_ms']:.3f} "
              f"launches={st['last_launches']} Mcell-updates/s={n * args.steps / (st['last_ms'] / 1e3) / 1e6:.1f} "
              f"stats={st}")
        b.close()
        return
    if args.workload == "l256":
        sc = scenes.l256()
    elif args.workload == "l256mur":  # the L256 grid closed by Mur faces instead of UPML
        from .fdtd import BC_MUR
        sc = scenes.l256()
        sc.set_boundary([BC_MUR] * 6, [0] * 6)
    elif args.workload == "l160":
        sc = scenes.l256(cells=160)
    elif args.workload == "p64":
        sc = scenes.p64()
    else:
        sc = scenes.d192()
    t0 = time.perf_counter()
    op = Operator(sc)
    cop = CompressedOperator(op)
    eng = Engine(cop, use_graphs=args.graphs, tile_y=args.tile_y, x_chunk=args.x_chunk)
    t1 = time.perf_counter()
    eng.iterate(args.steps)
    ms, launches = eng.last_timing()
    n = op.num_nodes
    print(f"{args.workload}: nodes={n} setup={t1 - t0:.2f}s steps={args.steps} device_ms={ms:.3f} "
          f"launches={launches} Mcell-updates/s={n * args.steps / (ms / 1e3) / 1e6:.1f} stats={eng.stats()}")
    eng.close()


if __name__ == "__main__":
    main()
