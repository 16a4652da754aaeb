"""wipems_gb300 -- GB300-native FDTD engine for openEMS-style simulations.

The Yee E/H time stepping with fused UPML, Lorentz/Drude ADE, excitation and
on-device probes runs in hand-written sm_103a CUDA kernels
(csrc/kernels.cuh), behind the C ABI of include/wipems_fdtd.h.  The host
operator build (csrc/operator.cpp) restates openEMS's Operator.
"""
from .fdtd import (BC_PEC, BC_PMC, BC_PML, C0, EPS0, MUE0, Batch, CompressedOperator, Engine, Operator, Samples,
                   Scene, SceneSpec, Server, run_fdtd)

__all__ = ["Scene", "SceneSpec", "Operator", "CompressedOperator", "Batch", "Server", "Engine", "Samples", "run_fdtd", "BC_PEC", "BC_PMC", "BC_PML", "EPS0", "MUE0",
           "C0"]
