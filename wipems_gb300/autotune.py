"""Autotuner for the half-step kernels.  Single jobs: the tile height (4- or
8-row tiles of 32 z-nodes), the TMA ring depth (stages) and the x-chunk
(planes per block); batches: the x-chunk, the CUDA-graph length and the
resident blocks per SM of the persistent kernels (how many work items each
SM holds at once).  Every candidate is timed the way the engine runs it,
with CUDA events on the engine's stream.

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
DEFAULT_TILE_Y = (4, 8)


def _cache_path() -> Path:
    p = os.environ.get("WIPEMS_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "wipems_gb300" / "tune.json"


def signature(cop) -> str:
    i = cop.info
    n = i["num_lines"]
    return (f"{n[0]}x{n[1]}x{n[2]}_u{int(i['num_upml_nodes'] > 0)}_a{int(i['num_ade_nodes'] > 0)}"
            f"_i{i['index_bytes_e']}{i['index_bytes_h']}_g{i['geometry_factored']}_r{i.get('rotation', 0)}")


def tune(cop, stages=DEFAULT_STAGES, xchunks=DEFAULT_XCHUNK, steps: int = 30, device: int = 0, verbose=False,
         kernels=("tma",), tile_ys=DEFAULT_TILE_Y):
    """Times every (kernel, tile_y, stages, x_chunk) combination the way the
    engine runs -- CUDA-graph chunks of one probe interval, device time from
    CUDA events over `steps` timesteps -- and returns (best, table), best
    minimising the time per timestep.  kernels may add "fused" (the
    single-pass kernel, where the grid allows it; its tile is fixed)."""
    from ._abi import FdtdError
    from .fdtd import Engine
    table = []
    for k in kernels:
        for ty in (tile_ys if k == "tma" else (0,)):
            for s in stages:
                for xc in xchunks:
                    try:
                        eng = Engine(cop, device=device, stages=s, x_chunk=xc, max_timesteps=2 * steps + 64,
                                     kernel=k, tile_y=ty)
                    except FdtdError:
                        break  # kernel not applicable to this grid
                    eng.iterate(min(steps, 16))  # warm-up, graph instantiation
                    eng.reset()
                    eng.iterate(steps)
                    ms, _ = eng.last_timing()
                    tile = eng.stats()["tile_y"]
                    eng.close()
                    table.append(dict(kernel=k, tile_y=tile, stages=s, x_chunk=xc, ms_step=ms / steps))
                    if verbose:
                        print(f"kernel={k:5s} tile_y={tile} stages={s} x_chunk={xc:3d}  {ms / steps * 1e3:8.1f} us/step",
                              flush=True)
    best = min(table, key=lambda r: r["ms_step"])
    return best, table


def tune_batch(cops, xchunks=(16, 32, 64), graph_steps=(32,), blocks_per_sm=(0, 3, -1), chains=(1, 2, 4),
               tile_ys=(8, 4), steps: int = 64, device: int = 0, verbose=False):
    """Batched mode: times the batch's kernels over the whole job set for
    every (tile_y, x_chunk, graph_steps, blocks_per_sm, chains) combination
    over `steps` timesteps (fresh engines per candidate, device time from
    CUDA events); blocks_per_sm caps the resident blocks each SM runs (0 = as
    many as fit; -1 = no persistent blocks, one block per work item) and
    chains splits each kernel-variant group into job ranges advancing on
    their own streams -- the tile shape and the jobs-per-SM schedule of the
    work list.  Chains and 4-row tiles are tried with the non-persistent
    kernels only (persistent grids each fill the GPU).  Returns (best, table)."""
    from .fdtd import Batch, Engine
    table = []
    for bps in blocks_per_sm:
        for ty in (tile_ys if bps < 0 else (8,)):
            for ch in (chains if bps < 0 else (1,)):
                for xc in xchunks:
                    for gs in graph_steps:
                        engines = [Engine(c, device=device, max_timesteps=steps + 4 * gs, kernel="tma") for c in cops]
                        b = Batch(engines, x_chunk=xc, graph_steps=gs, blocks_per_sm=bps, chains=ch, tile_y=ty)
                        b.iterate(gs)  # warm-up, graph instantiation
                        n = max(gs, steps // gs * gs)
                        b.iterate(n)
                        st = b.stats()
                        ms = st["last_ms"] / n
                        b.close()
                        for e in engines:
                            e.close()
                        table.append(dict(x_chunk=xc, graph_steps=gs, blocks_per_sm=bps, chains=ch, tile_y=ty,
                                          persistent_blocks=st["persistent_blocks"], ms_per_step=ms))
                        if verbose:
                            print(f"blocks_per_sm={bps} tile_y={ty} chains={ch} x_chunk={xc:3d} graph_steps={gs:3d}"
                                  f"  {ms * 1e3:8.1f} us/step", flush=True)
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
