"""ORACLE -- test infrastructure only (imported by tests/, smoke() and the
CPU-baseline arm of bench.py; never by the product package).

Python wrapper of liboracle.so: the CPU restatement of the reference's
operator build (operator_oracle.cpp) and of its FP32 time stepping
(fdtd_oracle.cpp); see those files for the reference citations."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi
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
        L.oracle_operator_build.restype = C.c_int
        L.oracle_operator_build.argtypes = [C.POINTER(abi.OracleScene), C.c_int, C.POINTER(C.c_void_p)]
        L.oracle_operator_destroy.restype = None
        L.oracle_operator_destroy.argtypes = [C.c_void_p]
        L.oracle_operator_info.restype = C.c_int
        L.oracle_operator_info.argtypes = [C.c_void_p, C.POINTER(abi.OracleOpInfo)]
        L.oracle_operator_probe.restype = C.c_int
        L.oracle_operator_probe.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(abi.ProbeDesc)]
        L.oracle_operator_describe.restype = C.c_int
        L.oracle_operator_describe.argtypes = [C.c_void_p, C.POINTER(abi.OpDesc)]
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


_KIND = {"material": 1, "metal": 2, "lumped": 3, "excitation": 4, "probe": 5}


def _scene_struct(spec: dict):
    """ctypes scene input from a scene's recorded inputs (Scene.spec)."""
    keep = []
    sc = abi.OracleScene()
    for a in range(3):
        l = np.ascontiguousarray(spec["lines"][a], np.float64)
        keep.append(l)
        sc.lines[a] = l.ctypes.data_as(C.POINTER(C.c_double))
        sc.num_lines[a] = len(l)
    sc.unit = spec["unit"]
    sc.bg_eps, sc.bg_mue, sc.bg_kappa, sc.bg_sigma = spec["background"]
    for k in range(6):
        sc.bc[k] = spec["bc"][k]
        sc.pml_size[k] = spec["pml_size"][k]
        sc.mur_vph[k] = spec["mur_vph"][k]
    sc.f0, sc.fc = spec["f0"], spec["fc"]
    sc.excite_type = spec.get("excite_type", 0)
    sc.f_max = spec.get("f_max", 0.0)
    fn = spec.get("function", "").encode()
    keep.append(fn)
    sc.function = fn
    sc.nr_ts = spec["nr_ts"]
    sc.oversampling = spec["oversampling"]
    prims = (abi.OraclePrim * max(1, len(spec["prims"])))()
    for i, p in enumerate(spec["prims"]):
        q = prims[i]
        q.kind = _KIND[p["kind"]]
        q.priority = p["priority"]
        for a in range(3):
            q.start[a], q.stop[a] = p["start"][a], p["stop"][a]
        q.eps, q.kappa, q.mue, q.sigma = (p.get(k, d) for k, d in (("eps", 1.0), ("kappa", 0.0), ("mue", 1.0),
                                                                  ("sigma", 0.0)))
        q.disp_order = p.get("disp_order", 0)
        for name in ("eps_plasma_f", "eps_relax_t", "eps_pole_f", "mue_plasma_f", "mue_relax_t", "mue_pole_f"):
            for o, v in enumerate(p.get(name, [])):
                getattr(q, name)[o] = v
        q.ny = p.get("ny", 2)
        q.le_type = p.get("le_type", 0)
        q.R, q.C, q.L = p.get("R", -1.0), p.get("C", -1.0), p.get("L", -1.0)
        q.caps = p.get("caps", 0)
        q.exc_type = p.get("exc_type", 0)
        for a, v in enumerate(p.get("exc_vec", [0.0, 0.0, 0.0])):
            q.exc_vec[a] = v
        q.delay = p.get("delay", 0.0)
        q.probe_type = p.get("probe_type", 0)
        q.weight = p.get("weight", 1.0)
        q.norm_dir = p.get("norm_dir", -1)
    sc.num_prims = len(spec["prims"])
    sc.prims = prims
    keep.append(prims)
    return sc, keep


class Operator:
    """The oracle's own operator build from a scene's recorded inputs
    (Scene.spec): .desc (engine description, include/wipems_fdtd.h layout),
    .probes, .dT, .nyquist, .probe_interval, .num_lines -- the attributes of
    the product's Operator that oracle.run and the tests read."""

    def __init__(self, spec: dict, threads: int = 0):
        if spec is None:
            raise ValueError("the scene has no recorded inputs (scenes read from XML are not recorded)")
        sc, self._keep = _scene_struct(spec)
        h = C.c_void_p()
        rc = lib().oracle_operator_build(C.byref(sc), int(threads), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle_operator_build failed ({rc})")
        self._h = h
        info = abi.OracleOpInfo()
        lib().oracle_operator_info(h, C.byref(info))
        self.num_lines = tuple(int(x) for x in info.num_lines)
        self.dT = float(info.dT)
        self.nyquist = int(info.nyquist)
        self.probe_interval = int(info.probe_interval)
        self.signal_length = int(info.signal_length)
        self.max_excite_ts = int(info.max_excite_ts)
        self.desc = abi.OpDesc()
        lib().oracle_operator_describe(h, C.byref(self.desc))
        self.probes = []
        for i in range(info.num_probes):
            p = abi.ProbeDesc()
            lib().oracle_operator_probe(h, i, C.byref(p))
            self.probes.append(p)

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                lib().oracle_operator_destroy(self._h)
            except Exception:
                pass
            self._h = None


def _arr(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def desc_arrays(desc) -> dict:
    """Every array and scalar of an engine description (either the product's
    or the oracle's) as numpy arrays keyed by name, for bitwise comparison."""
    N = tuple(int(x) for x in desc.num_lines)
    nn = 3 * N[0] * N[1] * N[2]
    out = {"num_lines": np.array(N), "dT": np.array([desc.dT])}
    for k in ("vv", "vi", "ii", "iv"):
        out[k] = _arr(getattr(desc, k), nn, np.float32)
    for s in range(desc.num_upml):
        u = desc.upml[s]
        nl = tuple(int(x) for x in u.num_lines)
        out[f"upml{s}.box"] = np.array(list(u.start) + list(nl))
        for k in ("vv", "vvfo", "vvfn", "ii", "iifo", "iifn"):
            out[f"upml{s}.{k}"] = _arr(getattr(u, k), 3 * nl[0] * nl[1] * nl[2], np.float32)
    for o in range(desc.num_ade_orders):
        a = desc.ade[o]
        c = int(a.count)
        out[f"ade{o}.flags"] = np.array([c, a.volt_on, a.curr_on, a.volt_lor_on, a.curr_lor_on])
        for n in range(3):
            out[f"ade{o}.pos{n}"] = _arr(a.pos[n], c, np.uint32)
        for k in ("v_int", "v_ext", "v_lor", "i_int", "i_ext", "i_lor"):
            out[f"ade{o}.{k}"] = _arr(getattr(a, k), 3 * c, np.float32)
    for side in ("volt", "curr"):
        c = int(getattr(desc, side + "_count"))
        for n in range(3):
            out[f"{side}.index{n}"] = _arr(getattr(desc, side + "_index")[n], c, np.uint32)
        out[f"{side}.dir"] = _arr(getattr(desc, side + "_dir"), c, np.uint16)
        out[f"{side}.amp"] = _arr(getattr(desc, side + "_amp"), c, np.float32)
        out[f"{side}.delay"] = _arr(getattr(desc, side + "_delay"), c, np.uint32)
    L = int(desc.signal_length)
    out["signal_volt"] = _arr(desc.signal_volt, L, np.float32)
    out["signal_curr"] = _arr(desc.signal_curr, L, np.float32)
    out["signal_period_ts"] = np.array([desc.signal_period_ts])
    for f in range(desc.num_mur):
        m = desc.mur[f]
        out[f"mur{f}.geom"] = np.array([m.ny, m.top, m.line, m.shift, m.n_p, m.n_pp, m.start_ts])
        out[f"mur{f}.coef_p"] = _arr(m.coef_p, m.n_p * m.n_pp, np.float32)
        out[f"mur{f}.coef_pp"] = _arr(m.coef_pp, m.n_p * m.n_pp, np.float32)
    if desc.rlc:
        r = desc.rlc[0]
        c = int(r.count)
        for n in range(3):
            out[f"rlc.pos{n}"] = _arr(r.pos[n], c, np.uint32)
        out["rlc.dir"] = _arr(r.dir, c, np.int32)
        for k in ("ilv", "i2v", "vv2", "vj1", "vj2", "vvd", "ib0", "b1", "b2"):
            out[f"rlc.{k}"] = _arr(getattr(r, k), c, np.float32)
    return out


def probe_tuples(probes) -> list:
    """Snapped probes as comparable tuples."""
    return [(p.type, tuple(p.start), tuple(p.stop), tuple(p.start_inside), tuple(p.stop_inside), p.norm_dir,
             p.weight, p.enabled) for p in probes]
