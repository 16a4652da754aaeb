"""Autotuner for the half-step kernels: picks the TMA ring depth (stages) and
the x-chunk (planes per block) of a workload by timing each candidate with
CUDA events on the engine stream (Engine.profile_kernels).

    python -m wipems_gb300.autotune --workload l256

Results are cached per workload signature (grid, features, index width) in
$WIPEMS_TUNE_CACHE (default ~/.cache/wipems_gb300/tune.json).
"""
from __future__ import annotations

import argparse
import json
import os
from pathlib import Path

DEFAULT_STAGES = (3, 4)
DEFAULT_XCHUNK = (1, 2, 4, 8, 16)


def _cache_path() -> Path:
    p = os.environ.get("WIPEMS_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "wipems_gb300" / "tune.json"


def signature(cop) -> str:
    i = cop.info
    n = i["num_lines"]
    return (f"{n[0]}x{n[1]}x{n[2]}_u{int(i['num_upml_nodes'] > 0)}_a{int(i['num_ade_nodes'] > 0)}"
            f"_i{i['index_bytes_e']}{i['index_bytes_h']}_g{i['geometry_factored']}")


def tune(cop, stages=DEFAULT_STAGES, xchunks=DEFAULT_XCHUNK, steps: int = 30, device: int = 0, verbose=False,
         kernels=("tma",)):
    """Times every (kernel, stages, x_chunk) combination the way the engine
    runs -- CUDA-graph chunks of one probe interval, device time from CUDA
    events over `steps` timesteps -- and returns (best, table), best
    minimising the time per timestep.  kernels may add "fused" (the
    single-pass kernel, where the grid allows it)."""
    from ._abi import FdtdError
    from .fdtd import Engine
    table = []
    for k in kernels:
        for s in stages:
            for xc in xchunks:
                try:
                    eng = Engine(cop, device=device, stages=s, x_chunk=xc, max_timesteps=2 * steps + 64, kernel=k)
                except FdtdError:
                    break  # kernel not applicable to this grid
                eng.iterate(min(steps, 16))  # warm-up, graph instantiation
                eng.reset()
                eng.iterate(steps)
                ms, _ = eng.last_timing()
                eng.close()
                table.append(dict(kernel=k, stages=s, x_chunk=xc, ms_step=ms / steps))
                if verbose:
                    print(f"kernel={k:5s} stages={s} x_chunk={xc:3d}  {ms / steps * 1e3:8.1f} us/step", flush=True)
    best = min(table, key=lambda r: r["ms_step"])
    return best, table


def tune_batch(cops, xchunks=(8, 16), graph_steps=(8, 32), steps: int = 64, device: int = 0, verbose=False):
    """Batched mode: times the persistent kernels of the whole job set for
    every (x_chunk, graph_steps) pair over `steps` timesteps (fresh engines
    per candidate, device time from CUDA events); returns (best, table)."""
    from .fdtd import Batch, Engine
    table = []
    for xc in xchunks:
        for gs in graph_steps:
            engines = [Engine(c, device=device, max_timesteps=steps + 4 * gs, kernel="tma") for c in cops]
            b = Batch(engines, x_chunk=xc, graph_steps=gs)
            b.iterate(gs)  # warm-up, graph instantiation
            n = max(gs, steps // gs * gs)
            b.iterate(n)
            ms = b.stats()["last_ms"] / n
            b.close()
            for e in engines:
                e.close()
            table.append(dict(x_chunk=xc, graph_steps=gs, ms_per_step=ms))
            if verbose:
                print(f"x_chunk={xc:3d} graph_steps={gs:3d}  {ms * 1e3:8.1f} us/step", flush=True)
    best = min(table, key=lambda r: r["ms_per_step"])
    return best, table


def cached(cop):
    """Best (stages, x_chunk) from the cache, or None."""
    p = _cache_path()
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
    except (OSError, ValueError):
        return None
    return d.get(signature(cop))


def store(cop, best):
    p = _cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        d = json.loads(p.read_text()) if p.exists() else {}
        d[signature(cop)] = best
        p.write_text(json.dumps(d, indent=1))
    except OSError:
        pass


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="l256", choices=["l256", "l160", "d192", "p64"])
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--fused", action="store_true", help="also time the single-pass kernel")
    args = ap.parse_args()
    from . import CompressedOperator, Operator, scenes
    sc = {"l256": lambda: scenes.l256(), "l160": lambda: scenes.l256(cells=160), "d192": lambda: scenes.d192(),
          "p64": lambda: scenes.p64()}[args.workload]()
    op = Operator(sc)
    cop = CompressedOperator(op)
    best, table = tune(cop, steps=args.steps, verbose=True, kernels=("tma", "fused") if args.fused else ("tma",))
    n = op.num_nodes
    print("best", json.dumps(best), f"Mcell-updates/s={n / (best['ms_step'] / 1e3) / 1e6:.0f}")
    store(cop, best)


if __name__ == "__main__":
    main()
