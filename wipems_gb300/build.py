"""In-tree build of libwipems_fdtd.so (CUDA engine + host operator) for sm_103a.

The library is compiled with plain nvcc / g++ calls (no torch extension and
no cmake) into wipems_gb300/_build/.  Translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libwipems_fdtd.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-fmad=false", "-Xptxas", "-v"]
# host code: no FMA contraction (the operator's float/double expressions are
# rounded in the reference's order); -fno-math-errno only drops the errno
# side effect of sqrt & co. (values unchanged), which lets loops such as the
# timestep search vectorize
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-math-errno", "-pthread",
             "-I/usr/local/cuda/include"]

CU_SOURCES = ["engine.cu", "engine_adex.cu", "energy_static.cu", "batch.cu"]
CXX_SOURCES = ["operator.cpp", "compress.cpp", "server.cpp", "xml_scene.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA engine cannot be built")


def _sources() -> list[Path]:
    out = []
    for name in CU_SOURCES + CXX_SOURCES:
        p = SRC / name
        if p.exists():
            out.append(p)
    return out


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(SRC.glob("*")) + [INCLUDE / "wipems_fdtd.h", Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the engine library if any source is newer than it."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    procs = []
    objs = []
    for src in _sources():
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if src.suffix == ".cu":
            cmd = [nvcc, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        else:
            cmd = [cxx, *CXX_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        log = BUILD / (src.stem + ".log")
        procs.append((cmd, subprocess.Popen(cmd, stdout=open(log, "w"), stderr=subprocess.STDOUT), log))
    failed = []
    for cmd, p, log in procs:
        if p.wait() != 0:
            failed.append((cmd, log.read_text()))
        elif verbose:
            sys.stderr.write(log.read_text())
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + out for c, out in failed)
        raise RuntimeError("build of libwipems_fdtd.so failed:\n" + msg)
    tmp = BUILD / "libwipems_fdtd.so.tmp"
    link = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link of libwipems_fdtd.so failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
