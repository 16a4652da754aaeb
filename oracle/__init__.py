"""ORACLE -- test infrastructure only (imported by tests/, smoke() and the
CPU-baseline arm of bench.py; never by the product package).

Python wrapper of liboracle.so, the CPU restatement of the reference's FP32
time stepping (see fdtd_oracle.cpp for the reference citations)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIB
from .build import build as build_lib

_lib = None

BASIC = 0          # Engine (FDTD/engine.cpp)
SSE_COMPRESSED_MT = 1  # Engine_SSE_Compressed + Engine_Multithread


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build_lib()
        L = C.CDLL(str(LIB))
        L.oracle_run.restype = C.c_long
        L.oracle_run.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_uint, C.c_uint, C.c_int, C.c_int, C.c_int,
                                 C.POINTER(C.c_double), C.c_long, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                 C.POINTER(C.c_double)]
        _lib = L
    return _lib


def run(desc, probes, n_steps: int, interval: int, engine: int = BASIC, threads: int = 1, energy: bool = True,
        fields: bool = True):
    """Runs the oracle on an fdtd_op_desc (ctypes structure) and a sequence
    of fdtd_probe_desc structures.  Returns dict(ts, energy, values, volt,
    curr, seconds)."""
    nl = tuple(int(x) for x in desc.num_lines)
    nprobe = len(probes)
    ProbeArr = type(probes[0]) * nprobe if nprobe else None
    parr = ProbeArr(*probes) if nprobe else None
    max_rows = (n_steps // interval + 2) if interval else 0
    row = 2 + sum(3 if p.type in (2, 3) else 1 for p in probes)  # three columns per field probe
    samples = np.zeros((max(max_rows, 1), row), np.float64)
    shape = (3,) + nl
    V = np.zeros(shape, np.float32) if fields else None
    I = np.zeros(shape, np.float32) if fields else None
    secs = C.c_double()
    rows = lib().oracle_run(C.addressof(desc), C.addressof(parr) if nprobe else None, nprobe, int(n_steps),
                            int(interval), int(engine), int(threads), int(energy),
                            samples.ctypes.data_as(C.POINTER(C.c_double)), max_rows,
                            V.ctypes.data_as(C.POINTER(C.c_float)) if fields else None,
                            I.ctypes.data_as(C.POINTER(C.c_float)) if fields else None, C.byref(secs))
    if rows < 0:
        raise RuntimeError("oracle_run failed")
    s = samples[:rows]
    return dict(ts=s[:, 0].astype(np.int64), energy=s[:, 1], values=s[:, 2:], volt=V, curr=I,
                seconds=secs.value)
