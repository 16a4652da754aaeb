"""Builds the oracle (CPU restatements of the reference's operator build and
time stepping) into oracle/_build/liboracle.so.  Test infrastructure only.

The reference itself is not compiled: its engine sources include CSXCAD,
Boost and fparser headers (FDTD/operator.h, FDTD/engine_sse_compressed.cpp,
FDTD/excitation.cpp), none of which exist in this image.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SRCS = [HERE / "fdtd_oracle.cpp", HERE / "operator_oracle.cpp"]
HDR = HERE.parent / "include" / "wipems_fdtd.h"

# -ffp-contract=off: no FMA contraction (the reference's x86-64 build has none).
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists():
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in (*SRCS, HDR, Path(__file__))):
            return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = BUILD / "liboracle.so.tmp"
    cmd = [os.environ.get("CXX", "g++"), *FLAGS, "-o", str(tmp), *[str(p) for p in SRCS]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
