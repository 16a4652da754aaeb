"""The reference-side glue (wipems_gb300/openems/): Operator_CUDA,
Engine_CUDA and Engine_Interface_CUDA, written against openEMS's Operator /
Engine / Engine_Interface_FDTD (FDTD/operator.h:55, FDTD/engine.h:42-79,
FDTD/engine_interface_fdtd.h), and the bridge that flattens an operator's
pointer trees into the engine description.

- The glue compiles to object code against the reference's own headers
  (with compile-time stand-ins for the CSXCAD and Boost declarations those
  headers name), where the reference tree is present.
- The bridge, fed pointer trees laid out as openEMS lays them out (one
  allocation per z-line), reproduces the engine description bit for bit on
  every feature; on the GPU the engine built from that description steps
  exactly like the oracle."""
import ctypes as C
import os
import subprocess
from pathlib import Path

import pytest

import oracle
from wipems_gb300 import CompressedOperator, Engine, Operator, _abi, scenes

from helpers import oracle_inputs

pytestmark = pytest.mark.usefixtures("libs")

ROOT = Path(__file__).resolve().parents[1]
GLUE = ROOT / "wipems_gb300" / "openems"
STUBS = Path(__file__).parent / "openems_stubs"
BUILD = Path(__file__).parent / "glue" / "_build"
REFERENCE = Path(os.environ.get("WIPEMS_OPENEMS_SOURCE", "/root/reference"))


@pytest.mark.skipif(not (REFERENCE / "FDTD" / "operator.h").exists(), reason="openEMS sources not present")
@pytest.mark.parametrize("unit", ["operator_cuda", "engine_cuda", "engine_interface_cuda"])
def test_glue_compiles_against_the_reference_headers(unit, tmp_path):
    cmd = ["g++", "-std=c++17", "-c", "-O1", "-Wall", "-Werror=return-type", f"-I{STUBS}", f"-I{REFERENCE}",
           f"-I{REFERENCE / 'FDTD'}", f"-I{REFERENCE / 'tools'}", f"-I{ROOT / 'include'}", str(GLUE / f"{unit}.cpp"),
           "-o", str(tmp_path / f"{unit}.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def _harness():
    BUILD.mkdir(parents=True, exist_ok=True)
    so = BUILD / "libbridge_harness.so"
    src = Path(__file__).parent / "glue" / "bridge_harness.cpp"
    deps = [src, GLUE / "openems_bridge.h", ROOT / "include" / "wipems_fdtd.h"]
    if not so.exists() or any(d.stat().st_mtime > so.stat().st_mtime for d in deps):
        tmp = BUILD / "libbridge_harness.so.tmp"
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-o", str(tmp), str(src)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        os.replace(tmp, so)
    L = C.CDLL(str(so))
    L.bridge_build.restype = C.c_void_p
    L.bridge_build.argtypes = [C.c_void_p]
    L.bridge_desc.restype = C.c_void_p
    L.bridge_desc.argtypes = [C.c_void_p]
    L.bridge_free.argtypes = [C.c_void_p]
    return L


class BridgedOperator:
    """The product operator's description sent through openEMS-layout
    pointer trees and the bridge; quacks like wipems_gb300.Operator."""

    def __init__(self, op):
        self._L = _harness()
        self._h = self._L.bridge_build(C.addressof(op.desc))
        self.desc = _abi.FdtdOpDesc.from_address(self._L.bridge_desc(self._h))
        self.num_lines, self.probes, self.probe_interval, self.scene = op.num_lines, op.probes, op.probe_interval, op.scene
        self.dT = op.dT

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.bridge_free(self._h)
            self._h = None


CASES = ["upml", "graded", "drude", "lorentz", "mixed", "mur", "rlc", "rlc_mur", "magnetic"]


@pytest.mark.parametrize("kind", CASES)
def test_bridge_rebuilds_the_description_bitwise(kind):
    op = Operator(scenes.mini(kind))
    b = BridgedOperator(op)
    a, c = oracle.desc_arrays(op.desc), oracle.desc_arrays(b.desc)
    assert sorted(a) == sorted(c)
    for k in a:
        assert a[k].tobytes() == c[k].tobytes(), k


@pytest.mark.parametrize("seed", [0, 1, 5, 8, 10, 13, 200, 202, 204, 207, 209, 211])
def test_bridge_rebuilds_random_scenes_bitwise(seed):
    """The seeded random scenes (UPML per axis, Lorentz / Drude of both
    families and of order 2, Mur faces, lumped RLC) through openEMS-layout
    pointer trees and the bridge: the same description, array for array."""
    from test_random_gpu import random_scene, random_scene_ext
    op = Operator(random_scene_ext(seed) if seed >= 200 else random_scene(seed))
    b = BridgedOperator(op)
    a, c = oracle.desc_arrays(op.desc), oracle.desc_arrays(b.desc)
    assert sorted(a) == sorted(c)
    for k in a:
        assert a[k].tobytes() == c[k].tobytes(), k


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["upml", "mixed", "rlc_mur", "magnetic"])
def test_engine_from_the_bridged_description_matches_oracle(kind):
    from test_parity_gpu import compare
    op = Operator(scenes.mini(kind, nr_ts=300))
    b = BridgedOperator(op)
    cop = CompressedOperator(b, mode="exact")
    eng = Engine(cop)
    eng.iterate(300)
    ref = oracle.run(*oracle_inputs(op), 300, op.probe_interval, engine=oracle.BASIC)
    compare(op, eng, ref)
