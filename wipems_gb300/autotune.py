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
DEFAULT_XCHUNK = (4, 8, 16)


def _cache_path() -> Path:
    p = os.environ.get("WIPEMS_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "wipems_gb300" / "tune.json"


def signature(cop) -> str:
    i = cop.info
    n = i["num_lines"]
    return (f"{n[0]}x{n[1]}x{n[2]}_u{int(i['num_upml_nodes'] > 0)}_a{int(i['num_ade_nodes'] > 0)}"
            f"_i{i['index_bytes_e']}{i['index_bytes_h']}_g{i['geometry_factored']}")


def tune(cop, stages=DEFAULT_STAGES, xchunks=DEFAULT_XCHUNK, steps: int = 30, device: int = 0, verbose=False):
    """Times every (stages, x_chunk) pair; returns (best, table) where best
    minimises the sum of the two half-step kernel times."""
    from .fdtd import Engine
    table = []
    for s in stages:
        for xc in xchunks:
            eng = Engine(cop, device=device, stages=s, x_chunk=xc, probe_interval=0, max_timesteps=steps + 10)
            eng.profile_kernels(4)  # warm-up
            mv, mc = eng.profile_kernels(steps)
            eng.close()
            table.append(dict(stages=s, x_chunk=xc, ms_volt=mv, ms_curr=mc))
            if verbose:
                print(f"stages={s} x_chunk={xc:3d}  volt {mv * 1e3:7.1f} us  curr {mc * 1e3:7.1f} us  "
                      f"sum {(mv + mc) * 1e3:7.1f} us", flush=True)
    best = min(table, key=lambda r: r["ms_volt"] + r["ms_curr"])
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
    args = ap.parse_args()
    from . import CompressedOperator, Operator, scenes
    sc = {"l256": lambda: scenes.l256(), "l160": lambda: scenes.l256(cells=160), "d192": lambda: scenes.d192(),
          "p64": lambda: scenes.p64()}[args.workload]()
    op = Operator(sc)
    cop = CompressedOperator(op)
    best, table = tune(cop, steps=args.steps, verbose=True)
    n = op.num_nodes
    print("best", json.dumps(best), f"Mcell-updates/s={n / ((best['ms_volt'] + best['ms_curr']) / 1e3) / 1e6:.0f}")
    store(cop, best)


if __name__ == "__main__":
    main()
