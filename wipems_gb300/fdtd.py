"""Host-side mirror of openEMS's Operator / Engine interface for the CUDA engine.

    Scene     ContinuousStructure + the <FDTD> setup (mesh, boxes, boundary
              conditions, excitation signal, probes); SceneSpec is the
              same scene as plain data, without native code.
    Operator  Operator::CalcECOperator (FDTD/operator.cpp:973-1084) with the
              excitation, UPML and Lorentz extension builds, run in C++.
    Engine    Engine_CUDA: IterateTS / GetNumberOfTimesteps / GetVolt /
              GetCurr (FDTD/engine.h:39-61) on the GPU, probes and energy
              reduced on the device.
    run_fdtd  openEMS::RunFDTD's loop (openems.cpp:1241-1345): iterate in
              probe-interval chunks until NrTS or the energy end criterion.

All compute goes through libwipems_fdtd.so; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import check, lib

EPS0 = 8.85418781762e-12
MUE0 = 1.256637062e-6
C0 = 299792458.0

BC_PEC, BC_PMC, BC_MUR, BC_PML = 0, 1, 2, 3


def _d3(v) -> C.Array:
    a = (C.c_double * 3)(*[float(x) for x in v])
    return a


def _lorentz_families(*fams):
    """The six per-order lists of a Lorentz material (eps plasma, relax,
    pole; mue plasma, relax, pole), each padded with zeros to the
    dispersion order = the longer plasma-frequency list."""
    order = max(len(fams[0]), len(fams[3]))
    if not 1 <= order <= 4:
        raise ValueError("add_lorentz: 1..4 plasma frequencies per family")
    out = []
    for f in fams:
        f = [float(v) for v in f]
        if len(f) > order:
            raise ValueError("add_lorentz: more values than dispersion orders")
        out.append(f + [0.0] * (order - len(f)))
    return out


class SceneSpec:
    """A scene as plain data: the recorder of the Scene calls (mesh lines,
    background, boundaries, pulse, boxes) in call order, with no native
    code.  `spec` is what an independent operator build (a checker) reads;
    Scene adds the native scene of the engine library on top."""

    def __init__(self, lines_x, lines_y, lines_z, unit: float):
        self._lines = [np.ascontiguousarray(l, dtype=np.float64) for l in (lines_x, lines_y, lines_z)]
        self.unit = unit
        self.nr_ts = 0
        self.probes: list[dict] = []
        self.meta: dict = {}
        self.spec: dict | None = dict(lines=[l.copy() for l in self._lines], unit=float(unit),
                                      background=(1.0, 1.0, 0.0, 0.0), bc=[0] * 6, pml_size=[0] * 6,
                                      mur_vph=[0.0] * 6, f0=0.0, fc=0.0, nr_ts=0, oversampling=4, prims=[],
                                      excite_type=0, f_max=0.0)

    @property
    def lines(self):
        return self._lines

    def _record(self, **kv):
        if self.spec is not None:
            self.spec.update(kv)

    def _prim(self, kind, priority, start, stop, **kv):
        if self.spec is not None:
            self.spec["prims"].append(dict(kind=kind, priority=int(priority), start=[float(v) for v in start],
                                           stop=[float(v) for v in stop], **kv))

    def set_background(self, eps_r=1.0, mue_r=1.0, kappa=0.0, sigma=0.0):
        self._record(background=(float(eps_r), float(mue_r), float(kappa), float(sigma)))

    def set_boundary(self, bc, pml_size=(8,) * 6):
        """Boundary per face (xmin, xmax, ymin, ymax, zmin, zmax): BC_PEC,
        BC_PMC, BC_MUR or BC_PML, with pml_size the layers of each PML face
        (8 by default, openEMS's size for a bare PML code).  A face that is
        not PML counts as 8 layers, openEMS's default, which openEMS's UPML
        build still reads: in the grading of a UPML on the opposite face and
        in the extent of the y / z slabs."""
        self._record(bc=[int(x) for x in bc], pml_size=[int(x) for x in pml_size])

    def set_mur_velocity(self, v_phase):
        """Mur phase velocity per face (m/s, 0 = from the boundary material)."""
        self._record(mur_vph=[float(x) for x in v_phase])

    def set_gauss_excite(self, f0: float, fc: float, nr_ts: int):
        self.nr_ts = int(nr_ts)
        self._record(f0=float(f0), fc=float(fc), nr_ts=int(nr_ts), excite_type=0, f_max=0.0)

    def set_sinus_excite(self, f0: float, nr_ts: int):
        """Sinusoid of frequency f0 (openEMS SetSinusExcite); the operator
        shortens dT so that 1/f0 is a whole number of timesteps."""
        self.nr_ts = int(nr_ts)
        self._record(f0=float(f0), fc=0.0, nr_ts=int(nr_ts), excite_type=1, f_max=0.0)

    def set_dirac_excite(self, f_max: float, nr_ts: int):
        """Dirac pulse: 1 at timestep 1 (openEMS SetDiracExcite)."""
        self.nr_ts = int(nr_ts)
        self._record(f0=0.0, fc=0.0, nr_ts=int(nr_ts), excite_type=2, f_max=float(f_max))

    def set_step_excite(self, f_max: float, nr_ts: int):
        """Step: 1 from timestep 0 on (openEMS SetStepExcite)."""
        self.nr_ts = int(nr_ts)
        self._record(f0=0.0, fc=0.0, nr_ts=int(nr_ts), excite_type=3, f_max=float(f_max))

    def set_custom_excite(self, function: str, f0: float, nr_ts: int, f_max: float = 0.0):
        """Custom signal, an expression of t (openEMS SetCustomExcite),
        sampled for nr_ts timesteps; probes sample at f0's Nyquist rate."""
        self.nr_ts = int(nr_ts)
        self._record(f0=float(f0), fc=0.0, nr_ts=int(nr_ts), excite_type=10, f_max=float(f_max),
                     function=str(function))

    def set_oversampling(self, os_: int):
        self._record(oversampling=int(os_))

    def add_material(self, start, stop, eps_r=1.0, kappa=0.0, mue_r=1.0, sigma=0.0, priority=0):
        self._prim("material", priority, start, stop, eps=float(eps_r), kappa=float(kappa), mue=float(mue_r),
                   sigma=float(sigma))

    def add_metal(self, start, stop, priority=0):
        self._prim("metal", priority, start, stop)

    def add_lumped(self, start, stop, direction, R=-1.0, Cap=-1.0, caps=True, priority=0):
        self._prim("lumped", priority, start, stop, ny=int(direction), le_type=0, R=float(R), C=float(Cap), L=-1.0,
                   caps=int(bool(caps)))

    def add_lumped_rlc(self, start, stop, direction, R=-1.0, L=-1.0, Cap=-1.0, series=False, caps=True, priority=0,
                       le_type=None):
        """Lumped element with an inductance and/or the series type
        (CSPropLumpedElement; Operator_Ext_LumpedRLC): parallel R || L || C
        or, with series=True, R - L - C in series.  Values < 0 are "not
        given".  le_type overrides series with the raw LEtype (-1 invalid:
        the element is ignored, as the reference ignores it)."""
        t = (1 if series else 0) if le_type is None else int(le_type)
        self._prim("lumped", priority, start, stop, ny=int(direction), le_type=t, R=float(R), C=float(Cap),
                   L=float(L), caps=int(bool(caps)))

    def add_excitation(self, start, stop, vec, exc_type=0, delay=0.0, priority=0):
        self._prim("excitation", priority, start, stop, exc_type=int(exc_type), exc_vec=[float(v) for v in vec],
                   delay=float(delay))

    def add_lorentz(self, start, stop, eps_r=1.0, kappa=0.0, mue_r=1.0, sigma=0.0, plasma_f=(), relax_t=(),
                    pole_f=(), priority=0, mue_plasma_f=(), mue_relax_t=(), mue_pole_f=()):
        """CSPropLorentzMaterial box: plasma_f / relax_t / pole_f are the
        electric family (EpsilonPlasmaFrequency, EpsilonRelaxTime,
        EpsilonLorPoleFrequency), mue_* the magnetic one (MuePlasmaFrequency,
        MueRelaxTime, MueLorPoleFrequency), one value per dispersion order;
        a pole frequency of 0 is a Drude pole."""
        fam = _lorentz_families(plasma_f, relax_t, pole_f, mue_plasma_f, mue_relax_t, mue_pole_f)
        self._prim("material", priority, start, stop, eps=float(eps_r), kappa=float(kappa), mue=float(mue_r),
                   sigma=float(sigma), disp_order=len(fam[0]), eps_plasma_f=fam[0], eps_relax_t=fam[1],
                   eps_pole_f=fam[2], mue_plasma_f=fam[3], mue_relax_t=fam[4], mue_pole_f=fam[5])

    def add_probe(self, start, stop, ptype: int, weight=1.0, norm_dir=-1, name=""):
        """A voltage (0), current (1), E-field (2) or H-field (3) probe box.
        A voltage probe needs a line (one coordinate differing between start
        and stop); the operator skips any other voltage box, as openEMS does
        (openems.cpp:481-486), so it gets no sample column."""
        self._prim("probe", 0, start, stop, probe_type=int(ptype), weight=float(weight), norm_dir=int(norm_dir))
        if int(ptype) == 0 and sum(float(a) != float(b) for a, b in zip(start, stop)) != 1:
            return
        self.probes.append(dict(name=name or f"probe{len(self.probes)}", type=ptype))

    def add_lumped_port(self, start, stop, direction, R, excite=1.0, priority=5, name="port"):
        """openEMS python LumpedPort (python/openEMS/ports.py:143-185):
        parallel-R lumped element with caps, soft E excitation of
        -direction*excite, voltage probe along the centre line (weight -1)
        and current probe across the mid plane (weight = direction)."""
        start = np.asarray(start, dtype=float)
        stop = np.asarray(stop, dtype=float)
        ny = int(direction)
        sign = float(np.sign(stop[ny] - start[ny]))
        if R > 0:
            self.add_lumped(start, stop, ny, R=R, caps=True, priority=priority)
        elif R == 0:
            self.add_metal(start, stop, priority=priority)
        if excite != 0:
            vec = np.zeros(3)
            vec[ny] = -1 * sign * excite
            self.add_excitation(start, stop, vec, exc_type=0, priority=priority)
        u_start = 0.5 * (start + stop)
        u_start[ny] = start[ny]
        u_stop = 0.5 * (start + stop)
        u_stop[ny] = stop[ny]
        self.add_probe(u_start, u_stop, 0, weight=-1, name=name + "_ut")
        i_start = start.copy()
        i_start[ny] = 0.5 * (start[ny] + stop[ny])
        i_stop = stop.copy()
        i_stop[ny] = 0.5 * (start[ny] + stop[ny])
        self.add_probe(i_start, i_stop, 1, weight=sign, norm_dir=ny, name=name + "_it")


class Scene(SceneSpec):
    """Mesh + primitives; the stand-in for CSXCAD: rectilinear mesh lines and
    priority-ordered axis-aligned boxes of material, metal, lumped elements,
    excitations and probes, held by the engine library (fdtd_scene_*), which
    checks every call; the calls are also recorded as plain data (`spec`)."""

    def __init__(self, lines_x, lines_y, lines_z, unit: float):
        super().__init__(lines_x, lines_y, lines_z, unit)
        h = C.c_void_p()
        ptr = [l.ctypes.data_as(C.POINTER(C.c_double)) for l in self._lines]
        check(lib().fdtd_scene_create(ptr[0], len(self._lines[0]), ptr[1], len(self._lines[1]), ptr[2],
                                      len(self._lines[2]), float(unit), C.byref(h)), "fdtd_scene_create")
        self._h = h

    @classmethod
    def from_spec(cls, spec: "SceneSpec") -> "Scene":
        """The native scene of a recorded one (replays its calls)."""
        d = spec.spec
        s = cls(*d["lines"], d["unit"])
        s.set_background(*d["background"])
        s.set_boundary(d["bc"], d["pml_size"])
        if any(d["mur_vph"]):
            s.set_mur_velocity(d["mur_vph"])
        et = d.get("excite_type", 0)
        if et == 1:
            s.set_sinus_excite(d["f0"], d["nr_ts"])
        elif et in (2, 3):
            (s.set_dirac_excite if et == 2 else s.set_step_excite)(d["f_max"], d["nr_ts"])
        elif et == 10:
            s.set_custom_excite(d["function"], d["f0"], d["nr_ts"], d["f_max"])
        elif d["fc"] > 0:
            s.set_gauss_excite(d["f0"], d["fc"], d["nr_ts"])
        if d["oversampling"] != 4:
            s.set_oversampling(d["oversampling"])
        for p in d["prims"]:
            k = p["kind"]
            a, b, pr = p["start"], p["stop"], p["priority"]
            if k == "material" and p.get("disp_order", 0) > 0:
                s.add_lorentz(a, b, p["eps"], p["kappa"], p["mue"], p["sigma"], p["eps_plasma_f"], p["eps_relax_t"],
                              p["eps_pole_f"], priority=pr, mue_plasma_f=p.get("mue_plasma_f", ()),
                              mue_relax_t=p.get("mue_relax_t", ()), mue_pole_f=p.get("mue_pole_f", ()))
            elif k == "material":
                s.add_material(a, b, p["eps"], p["kappa"], p["mue"], p["sigma"], priority=pr)
            elif k == "metal":
                s.add_metal(a, b, priority=pr)
            elif k == "lumped":
                s.add_lumped_rlc(a, b, p["ny"], R=p["R"], L=p["L"], Cap=p["C"], caps=p["caps"], priority=pr,
                                 le_type=p["le_type"])
            elif k == "excitation":
                s.add_excitation(a, b, p["exc_vec"], p["exc_type"], p["delay"], priority=pr)
            elif k == "probe":
                s.add_probe(a, b, p["probe_type"], p["weight"], p["norm_dir"])
        s.probes = list(spec.probes)
        s.meta = dict(spec.meta)
        s.nr_ts = spec.nr_ts
        return s

    @classmethod
    def from_xml(cls, xml: str) -> "Scene":
        """A scene from an openEMS XML document (the text, or a path to the
        file): the subset fdtd_scene_load_xml covers.  The run settings are
        in .xml_info (nr_ts, end_crit, ...)."""
        h = C.c_void_p()
        inf = _abi.FdtdXmlInfo()
        if "<" in xml:
            check(lib().fdtd_scene_load_xml(xml.encode(), C.byref(h), C.byref(inf)), "fdtd_scene_load_xml")
        else:
            check(lib().fdtd_scene_load_xml_file(str(xml).encode(), C.byref(h), C.byref(inf)),
                  "fdtd_scene_load_xml_file")
        s = cls.__new__(cls)
        s._h = h
        s._lines = None
        s.unit = None
        s.nr_ts = int(inf.nr_ts)
        s.probes = []
        s.meta = {}
        s.spec = None
        s.xml_info = {k: getattr(inf, k) for k, _ in inf._fields_}
        return s

    def dumps(self) -> list:
        """The time-domain E / H field dumps of the scene (XML <DumpBox>):
        dicts of name, field ("E"/"H"), interp, file_type, start, stop (drawing
        units) and step, for wipems_gb300.dumps.FieldDump.from_spec."""
        n = C.c_uint32()
        check(lib().fdtd_scene_num_dumps(self._h, C.byref(n)), "fdtd_scene_num_dumps")
        out = []
        for k in range(n.value):
            d = _abi.FdtdSceneDump()
            check(lib().fdtd_scene_get_dump(self._h, k, C.byref(d)), "fdtd_scene_get_dump")
            out.append(dict(name=d.name.decode(), field="EH"[d.field], interp=("none", "node", "cell")[d.interp],
                            file_type=d.file_type, start=list(d.start), stop=list(d.stop), step=list(d.step)))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                lib().fdtd_scene_destroy(self._h)
            except Exception:
                pass
            self._h = None

    def set_background(self, eps_r=1.0, mue_r=1.0, kappa=0.0, sigma=0.0):
        check(lib().fdtd_scene_set_background(self._h, eps_r, mue_r, kappa, sigma), "set_background")
        super().set_background(eps_r, mue_r, kappa, sigma)

    def set_boundary(self, bc, pml_size=(8,) * 6):
        b = (C.c_int * 6)(*bc)
        s = (C.c_uint32 * 6)(*pml_size)
        check(lib().fdtd_scene_set_boundary(self._h, b, s), "set_boundary")
        super().set_boundary(bc, pml_size)

    def set_mur_velocity(self, v_phase):
        check(lib().fdtd_scene_set_mur_velocity(self._h, (C.c_double * 6)(*v_phase)), "set_mur_velocity")
        super().set_mur_velocity(v_phase)

    def set_gauss_excite(self, f0: float, fc: float, nr_ts: int):
        check(lib().fdtd_scene_set_gauss_excite(self._h, f0, fc, int(nr_ts)), "set_gauss_excite")
        super().set_gauss_excite(f0, fc, nr_ts)

    def set_sinus_excite(self, f0: float, nr_ts: int):
        check(lib().fdtd_scene_set_sinus_excite(self._h, f0, int(nr_ts)), "set_sinus_excite")
        super().set_sinus_excite(f0, nr_ts)

    def set_dirac_excite(self, f_max: float, nr_ts: int):
        check(lib().fdtd_scene_set_dirac_excite(self._h, f_max, int(nr_ts)), "set_dirac_excite")
        super().set_dirac_excite(f_max, nr_ts)

    def set_step_excite(self, f_max: float, nr_ts: int):
        check(lib().fdtd_scene_set_step_excite(self._h, f_max, int(nr_ts)), "set_step_excite")
        super().set_step_excite(f_max, nr_ts)

    def set_custom_excite(self, function: str, f0: float, nr_ts: int, f_max: float = 0.0):
        check(lib().fdtd_scene_set_custom_excite(self._h, str(function).encode(), float(f0), float(f_max),
                                                 int(nr_ts)), "set_custom_excite")
        super().set_custom_excite(function, f0, nr_ts, f_max)

    def set_oversampling(self, os_: int):
        check(lib().fdtd_scene_set_oversampling(self._h, int(os_)), "set_oversampling")
        super().set_oversampling(os_)

    def add_material(self, start, stop, eps_r=1.0, kappa=0.0, mue_r=1.0, sigma=0.0, priority=0):
        check(lib().fdtd_scene_add_material(self._h, int(priority), _d3(start), _d3(stop), eps_r, kappa, mue_r,
                                            sigma), "add_material")
        super().add_material(start, stop, eps_r, kappa, mue_r, sigma, priority)

    def add_metal(self, start, stop, priority=0):
        check(lib().fdtd_scene_add_metal(self._h, int(priority), _d3(start), _d3(stop)), "add_metal")
        super().add_metal(start, stop, priority)

    def add_lumped(self, start, stop, direction, R=-1.0, Cap=-1.0, caps=True, priority=0):
        check(lib().fdtd_scene_add_lumped(self._h, int(priority), _d3(start), _d3(stop), int(direction), float(R),
                                          float(Cap), int(bool(caps))), "add_lumped")
        super().add_lumped(start, stop, direction, R, Cap, caps, priority)

    def add_lumped_rlc(self, start, stop, direction, R=-1.0, L=-1.0, Cap=-1.0, series=False, caps=True, priority=0,
                       le_type=None):
        t = (1 if series else 0) if le_type is None else int(le_type)
        check(lib().fdtd_scene_add_lumped_rlc(self._h, int(priority), _d3(start), _d3(stop), int(direction), t,
                                              float(R), float(L), float(Cap), int(bool(caps))), "add_lumped_rlc")
        super().add_lumped_rlc(start, stop, direction, R, L, Cap, series, caps, priority, le_type)

    def add_excitation(self, start, stop, vec, exc_type=0, delay=0.0, priority=0):
        check(lib().fdtd_scene_add_excitation(self._h, int(priority), _d3(start), _d3(stop), int(exc_type),
                                              _d3(vec), float(delay)), "add_excitation")
        super().add_excitation(start, stop, vec, exc_type, delay, priority)

    def add_lorentz(self, start, stop, eps_r=1.0, kappa=0.0, mue_r=1.0, sigma=0.0, plasma_f=(), relax_t=(),
                    pole_f=(), priority=0, mue_plasma_f=(), mue_relax_t=(), mue_pole_f=()):
        fam = _lorentz_families(plasma_f, relax_t, pole_f, mue_plasma_f, mue_relax_t, mue_pole_f)
        order = len(fam[0])
        arr = [(C.c_double * max(order, 1))(*f) for f in fam]
        check(lib().fdtd_scene_add_lorentz_material(self._h, int(priority), _d3(start), _d3(stop), eps_r, kappa,
                                                    mue_r, sigma, order, *arr), "add_lorentz")
        super().add_lorentz(start, stop, eps_r, kappa, mue_r, sigma, plasma_f, relax_t, pole_f, priority,
                            mue_plasma_f, mue_relax_t, mue_pole_f)

    def add_probe(self, start, stop, ptype: int, weight=1.0, norm_dir=-1, name=""):
        check(lib().fdtd_scene_add_probe(self._h, int(ptype), _d3(start), _d3(stop), float(weight), int(norm_dir)),
              "add_probe")
        super().add_probe(start, stop, ptype, weight, norm_dir, name)


class Operator:
    """Operator::CalcECOperator + extension builds, run on the host."""

    def __init__(self, scene: Scene, threads: int = 0):
        if not isinstance(scene, Scene):  # a recorded scene: make its native twin
            scene = Scene.from_spec(scene)
        h = C.c_void_p()
        check(lib().fdtd_operator_build(scene._h, int(threads), C.byref(h)), "fdtd_operator_build")
        self._h = h
        self.scene = scene
        info = _abi.FdtdOperatorInfo()
        check(lib().fdtd_operator_get_info(h, C.byref(info)), "fdtd_operator_get_info")
        self.info = info
        self.num_lines = tuple(int(x) for x in info.num_lines)
        self.dT = float(info.dT)
        self.probe_interval = int(info.probe_interval)
        self.nyquist = int(info.nyquist)
        self.desc = _abi.FdtdOpDesc()
        check(lib().fdtd_operator_describe(h, C.byref(self.desc)), "fdtd_operator_describe")
        self.probes = []
        for i in range(info.num_probes):
            p = _abi.FdtdProbeDesc()
            check(lib().fdtd_operator_get_probe(h, i, C.byref(p)), "fdtd_operator_get_probe")
            self.probes.append(p)

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                lib().fdtd_operator_destroy(self._h)
            except Exception:
                pass
            self._h = None

    @property
    def num_nodes(self) -> int:
        n = self.num_lines
        return n[0] * n[1] * n[2]

    def coefficients(self):
        """Reference-form vv, vi, ii, iv as numpy views [3][Nx][Ny][Nz]."""
        shape = (3,) + self.num_lines
        cnt = 3 * self.num_nodes
        out = []
        for name in ("vv", "vi", "ii", "iv"):
            ptr = getattr(self.desc, name)
            out.append(np.ctypeslib.as_array(ptr, shape=(cnt,)).reshape(shape))
        return out

    def signals(self):
        n = self.desc.signal_length
        if n == 0:
            return np.zeros(0, np.float32), np.zeros(0, np.float32)
        return (np.ctypeslib.as_array(self.desc.signal_volt, shape=(n,)).copy(),
                np.ctypeslib.as_array(self.desc.signal_curr, shape=(n,)).copy())

    def excitation(self):
        d = self.desc
        n = d.volt_count
        if n == 0:
            return dict(index=np.zeros((3, 0), np.uint32), dir=np.zeros(0, np.uint16), amp=np.zeros(0, np.float32))
        idx = np.stack([np.ctypeslib.as_array(d.volt_index[a], shape=(n,)) for a in range(3)])
        return dict(index=idx.copy(), dir=np.ctypeslib.as_array(d.volt_dir, shape=(n,)).copy(),
                    amp=np.ctypeslib.as_array(d.volt_amp, shape=(n,)).copy())


@dataclass
class Samples:
    ts: np.ndarray
    values: np.ndarray      # [nsamples][nprobes]
    energy: np.ndarray
    dT: float
    probe_types: list = field(default_factory=list)

    def times(self, p: int) -> np.ndarray:
        """Sample times of column p: voltage and E-field probes at ts*dT,
        current and H-field probes on the dual time (ts+0.5)*dT
        (openems.cpp:520-526)."""
        dual = 0.5 if self.probe_types[p] in (1, 3) else 0.0
        return (self.ts + dual) * self.dT


class CompressedOperator:
    """Operator_SSE_Compressed::CompressOperator analogue, per node: the
    uint16/uint32 tuple index + coefficient tables in (pinned) host memory.
    Runs without a GPU."""

    MODES = {"auto": 0, "exact": 1, "factorized": 2}

    def __init__(self, op: Operator, mode: str = "auto", rotation: int | str = "auto"):
        """rotation: the device axes (fdtd_compress_rot): "auto", or r in
        0..2 for device axis a = the operator's axis (a + r) % 3."""
        h = C.c_void_p()
        rot = -1 if rotation == "auto" else int(rotation)
        check(lib().fdtd_compress_rot(C.byref(op.desc), self.MODES[mode], rot, C.byref(h)), "fdtd_compress")
        self._h = h
        self.op = op
        info = _abi.FdtdCopInfo()
        check(lib().fdtd_cop_get_info(h, C.byref(info)), "fdtd_cop_get_info")
        self.info = {k: (list(getattr(info, k)) if k in ("num_lines", "trim_e", "device_lines") else getattr(info, k))
                     for k, _ in info._fields_}
        self.factorized = bool(self.info["geometry_factored"])
        self.rotation = self.info["rotation"]

    def __del__(self):
        if getattr(self, "_h", None):
            try:
                lib().fdtd_cop_destroy(self._h)
            except Exception:
                pass
            self._h = None

    def expand(self):
        """Reference-form vv, vi, ii, iv and the E/H flag words rebuilt from
        the index and tables."""
        shape = (3,) + self.op.num_lines
        out = [np.empty(shape, np.float32) for _ in range(4)]
        fe = np.empty(self.op.num_lines, np.uint32)
        fh = np.empty(self.op.num_lines, np.uint32)
        check(lib().fdtd_cop_expand(self._h, *[a.ctypes.data_as(_abi.PF) for a in out], fe.ctypes.data_as(_abi.PU32),
                                    fh.ctypes.data_as(_abi.PU32)), "fdtd_cop_expand")
        return out + [fe, fh]

    def expand_ext(self, half: int):
        """The ADE and UPML coefficients of one half (0 = E, 1 = H) as the
        kernels apply them: two [9][Nx][Ny][Nz] arrays (int/ext/lor, and
        vvp/vvfo/vvfn or the current-side terms), zero where a node has none."""
        shape = (9,) + self.op.num_lines
        ade = np.empty(shape, np.float32)
        upml = np.empty(shape, np.float32)
        check(lib().fdtd_cop_expand_ext(self._h, int(half), ade.ctypes.data_as(_abi.PF), upml.ctypes.data_as(_abi.PF)),
              "fdtd_cop_expand_ext")
        return ade, upml

    def expand_ade(self, half: int, order: int):
        """The Lorentz/Drude ADE terms of one dispersion order (0..3) of one
        half as the kernels apply them: [9][Nx][Ny][Nz] (int/ext/lor)."""
        ade = np.empty((9,) + self.op.num_lines, np.float32)
        check(lib().fdtd_cop_expand_ade(self._h, int(half), int(order), ade.ctypes.data_as(_abi.PF)),
              "fdtd_cop_expand_ade")
        return ade


class Engine:
    """Engine_CUDA on one GPU.  op is an Operator (compressed here) or a
    CompressedOperator (upload only)."""

    def __init__(self, op, device: int = 0, max_timesteps: int = 0, probe_interval: int | None = None,
                 use_graphs: bool = True, energy_on_probe: bool = True, tile_y: int = 0, x_chunk: int = 0,
                 probes: bool = True, kernel: str = "auto", stages: int = 0, end_crit: float = 0.0):
        cop = op if isinstance(op, CompressedOperator) else None
        if cop is not None:
            op = cop.op
        self.op = op
        o = _abi.FdtdEngineOpts()
        o.device = device
        o.max_timesteps = int(max_timesteps or op.scene.nr_ts or 100000)
        o.probe_interval = int(op.probe_interval if probe_interval is None else probe_interval)
        o.use_graphs = int(use_graphs)
        o.energy_on_probe = int(energy_on_probe)
        o.tile_y = int(tile_y)
        o.x_chunk = int(x_chunk)
        kinds = {"auto": 0, "direct": 1, "fused": 2, "tma": 3}
        if kernel not in kinds:
            raise ValueError("kernel must be 'auto', 'tma', 'direct' or 'fused'")
        o.kernel = kinds[kernel]
        o.stages = int(stages)
        o.end_crit = float(end_crit)
        h = C.c_void_p()
        if cop is not None:
            check(lib().fdtd_engine_create_compressed(cop._h, C.byref(o), C.byref(h)), "fdtd_engine_create_compressed")
        else:
            check(lib().fdtd_engine_create(C.byref(op.desc), C.byref(o), C.byref(h)), "fdtd_engine_create")
        self._h = h
        self.interval = o.probe_interval
        self.probe_types = []
        if probes:
            for p in op.probes:
                check(lib().fdtd_engine_add_probe(h, C.byref(p), None), "fdtd_engine_add_probe")
                self.probe_types += [p.type] * (3 if p.type in (2, 3) else 1)  # one column per field component

    def close(self):
        if getattr(self, "_h", None):
            lib().fdtd_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self):
        """Engine::Reset + Init: zero fields/states, numTS = 0."""
        check(lib().fdtd_engine_reset(self._h), "fdtd_engine_reset")

    def iterate(self, n: int):
        check(lib().fdtd_engine_iterate(self._h, int(n)), "fdtd_engine_iterate")

    def set_frequencies(self, freqs, fd_interval: int | None = None):
        """Frequency-domain probe accumulation on the device at the given
        frequencies (Hz).  The default interval follows the reference's
        Processing::AddFrequency (processing.cpp:150-170): the operator's
        Nyquist number, lowered for frequencies above the excited band;
        frequencies too high for the timestep are dropped, as there."""
        dT = self.op.dT
        kept = []
        interval = int(self.op.nyquist)
        for f in freqs:
            nyq = int(np.floor(1.0 / f / 2.0 / dT)) if f > 0 else 2 ** 32 - 1  # CalcNyquistNum (tools/useful.cpp:30-36)
            if nyq == 0:
                continue
            interval = min(interval, nyq) if interval else nyq
            kept.append(float(f))
        if fd_interval is not None:
            interval = int(fd_interval)
        arr = np.asarray(kept, np.float64)
        check(lib().fdtd_engine_set_fd(self._h, arr.ctypes.data_as(_abi.PD), len(kept), int(interval)),
              "fdtd_engine_set_fd")
        self.fd_freqs = arr
        self.fd_interval = interval
        return arr

    def fd_results(self):
        """(values [probe][frequency] complex, samples accumulated)."""
        nf = len(getattr(self, "fd_freqs", []))
        npr = len(self.probe_types)
        buf = np.zeros((npr, nf, 2), np.float64)
        cnt = C.c_uint32()
        check(lib().fdtd_engine_read_fd(self._h, buf.ctypes.data_as(_abi.PD), C.byref(cnt)), "fdtd_engine_read_fd")
        return buf[..., 0] + 1j * buf[..., 1], cnt.value

    def dump_field(self, field: str = "E", interp: str = "node", start=(0, 0, 0), stop=None, step=(1, 1, 1)):
        """E (V/m) or H (A/m) at the current timestep on the mesh lines
        start + i * step (indices, both ends included) of a box, interpolated
        as the reference's field dumps do (interp "none", "node" or "cell");
        returns a float32 array [3][n0][n1][n2] (fdtd_engine_dump_field)."""
        kinds = {"E": 0, "H": 1}
        modes = {"none": 0, "node": 1, "cell": 2}
        if field not in kinds or interp not in modes:
            raise ValueError("field must be 'E' or 'H', interp 'none', 'node' or 'cell'")
        if stop is None:
            stop = tuple(n - 1 for n in self.op.num_lines)
        b = _abi.FdtdDumpBox(kinds[field], modes[interp], (C.c_uint32 * 3)(*start), (C.c_uint32 * 3)(*stop),
                             (C.c_uint32 * 3)(*step))
        num = (C.c_uint32 * 3)()
        check(lib().fdtd_engine_dump_field(self._h, C.byref(b), None, 0, num), "fdtd_engine_dump_field")
        out = np.empty((3, num[0], num[1], num[2]), np.float32)
        check(lib().fdtd_engine_dump_field(self._h, C.byref(b), out.ctypes.data_as(_abi.PF), out.size, num),
              "fdtd_engine_dump_field")
        return out

    def checkpoint(self) -> bytes:
        """All device state of the engine as bytes (fdtd_engine_checkpoint)."""
        size = C.c_uint64()
        check(lib().fdtd_engine_checkpoint(self._h, None, 0, C.byref(size)), "fdtd_engine_checkpoint")
        buf = C.create_string_buffer(size.value)
        check(lib().fdtd_engine_checkpoint(self._h, buf, size.value, C.byref(size)), "fdtd_engine_checkpoint")
        return buf.raw[:size.value]

    def restore(self, blob: bytes):
        """Loads a checkpoint of an engine made from the same operator."""
        check(lib().fdtd_engine_restore(self._h, blob, len(blob)), "fdtd_engine_restore")

    def iterate_async(self, n: int):
        """Queues n timesteps on the engine's stream and returns (wait())."""
        check(lib().fdtd_engine_iterate_async(self._h, int(n)), "fdtd_engine_iterate_async")

    def wait(self):
        check(lib().fdtd_engine_wait(self._h), "fdtd_engine_wait")

    @property
    def done(self) -> bool:
        """True once the device end criterion (end_crit) stopped the job."""
        v = C.c_int()
        check(lib().fdtd_engine_done(self._h, C.byref(v)), "fdtd_engine_done")
        return bool(v.value)

    @property
    def num_timesteps(self) -> int:
        v = C.c_uint32()
        check(lib().fdtd_engine_num_timesteps(self._h, C.byref(v)), "num_timesteps")
        return v.value

    def samples(self) -> Samples:
        n = C.c_uint32()
        check(lib().fdtd_engine_num_samples(self._h, C.byref(n)), "num_samples")
        n = n.value
        np_ = len(self.probe_types)
        ts = np.zeros(n, np.uint32)
        vals = np.zeros((n, max(np_, 1)), np.float64)
        en = np.zeros(n, np.float64)
        if n:
            check(lib().fdtd_engine_read_samples(self._h, 0, n, ts.ctypes.data_as(_abi.PU32),
                                                 vals.ctypes.data_as(_abi.PD), en.ctypes.data_as(_abi.PD)),
                  "read_samples")
        return Samples(ts=ts.astype(np.int64), values=vals[:, :np_], energy=en, dT=self.op.dT,
                       probe_types=list(self.probe_types))

    def energy(self) -> float:
        v = C.c_double()
        check(lib().fdtd_engine_energy(self._h, C.byref(v)), "energy")
        return v.value

    def fields(self):
        shape = (3,) + self.op.num_lines
        V = np.empty(shape, np.float32)
        I = np.empty(shape, np.float32)
        check(lib().fdtd_engine_get_fields(self._h, V.ctypes.data_as(_abi.PF), I.ctypes.data_as(_abi.PF)),
              "get_fields")
        return V, I

    def get_volt(self, n, x, y, z) -> float:
        v = C.c_float()
        check(lib().fdtd_engine_get_volt(self._h, n, x, y, z, C.byref(v)), "get_volt")
        return v.value

    def set_volt(self, n, x, y, z, value: float):
        check(lib().fdtd_engine_set_volt(self._h, n, x, y, z, float(value)), "fdtd_engine_set_volt")

    def set_curr(self, n, x, y, z, value: float):
        check(lib().fdtd_engine_set_curr(self._h, n, x, y, z, float(value)), "fdtd_engine_set_curr")

    def probe_now(self, probe) -> float:
        """The unweighted integral of a voltage / current probe descriptor on
        the current fields (fdtd_engine_probe_now)."""
        v = C.c_double()
        check(lib().fdtd_engine_probe_now(self._h, C.byref(probe), C.byref(v)), "fdtd_engine_probe_now")
        return v.value

    def get_curr(self, n, x, y, z) -> float:
        v = C.c_float()
        check(lib().fdtd_engine_get_curr(self._h, n, x, y, z, C.byref(v)), "get_curr")
        return v.value

    def stats(self) -> dict:
        s = _abi.FdtdEngineStats()
        check(lib().fdtd_engine_get_stats(self._h, C.byref(s)), "get_stats")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def profile_kernels(self, n: int):
        """Mean device ms of one voltage and one current kernel launch over
        n timesteps (CUDA events on the engine stream)."""
        a = C.c_double()
        b = C.c_double()
        check(lib().fdtd_engine_profile_kernels(self._h, int(n), C.byref(a), C.byref(b)), "profile_kernels")
        return a.value, b.value

    def num_samples(self) -> int:
        n = C.c_uint32()
        check(lib().fdtd_engine_num_samples(self._h, C.byref(n)), "num_samples")
        return n.value

    def read_samples(self, first: int, count: int):
        np_ = len(self.probe_types)
        ts = np.zeros(count, np.uint32)
        vals = np.zeros((count, max(np_, 1)), np.float64)
        en = np.zeros(count, np.float64)
        if count:
            check(lib().fdtd_engine_read_samples(self._h, first, count, ts.ctypes.data_as(_abi.PU32),
                                                 vals.ctypes.data_as(_abi.PD), en.ctypes.data_as(_abi.PD)),
                  "read_samples")
        return ts, vals[:, :np_], en

    def last_timing(self):
        ms = C.c_double()
        n = C.c_uint64()
        check(lib().fdtd_engine_last_timing(self._h, C.byref(ms), C.byref(n)), "last_timing")
        return ms.value, n.value


class Batch:
    """Batched mode: the given engines advance together, one persistent
    kernel per half-step and kernel variant (see fdtd_batch_create).  The
    engines must outlive the batch."""

    def __init__(self, engines, x_chunk: int = 0, stages: int = 0, blocks_per_sm: int = 0, graph_steps: int = 0,
                 bin_mib: int = 0, chains: int = 0, tile_y: int = 0):
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e._h.value for e in self.engines])
        o = _abi.FdtdBatchOpts(int(x_chunk), int(stages), int(blocks_per_sm), int(graph_steps), int(bin_mib),
                               int(chains), int(tile_y))
        h = C.c_void_p()
        check(lib().fdtd_batch_create(arr, len(self.engines), C.byref(o), C.byref(h)), "fdtd_batch_create")
        self._h = h

    def iterate(self, n: int):
        check(lib().fdtd_batch_iterate(self._h, int(n)), "fdtd_batch_iterate")

    def stats(self) -> dict:
        s = _abi.FdtdBatchStats()
        check(lib().fdtd_batch_info(self._h, C.byref(s)), "fdtd_batch_info")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().fdtd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


JOB_STATES = ("queued", "building", "ready", "running", "done", "failed")


class Server:
    """Continuous-batching job server (fdtd_server_*): submit scenes at any
    time; operators are built on host worker threads, jobs are admitted by
    device footprint, advanced together in batched rounds and retired on
    their own end criterion."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, max_active: int = 0, round_steps: int = 0,
                 build_workers: int = 0, build_threads_per_job: int = 0, x_chunk: int = 0, stages: int = 0,
                 blocks_per_sm: int = 0, graph_steps: int = 0, bin_mib: int = 0, batch_min_jobs: int = 0,
                 tile_share: int = 0):
        o = _abi.FdtdServerOpts()
        o.device = device
        o.hbm_budget = int(hbm_budget)
        o.max_active = int(max_active)
        o.round_steps = int(round_steps)
        o.build_workers = int(build_workers)
        o.build_threads_per_job = int(build_threads_per_job)
        o.batch_min_jobs = int(batch_min_jobs)
        o.batch = _abi.FdtdBatchOpts(int(x_chunk), int(stages), int(blocks_per_sm), int(graph_steps), int(bin_mib))
        o.tile_share = int(tile_share)
        h = C.c_void_p()
        check(lib().fdtd_server_create(C.byref(o), C.byref(h)), "fdtd_server_create")
        self._h = h

    def submit(self, scene: Scene, end_crit: float = 0.0, max_timesteps: int = 0, probe_interval: int = 0,
               keep_fields: bool = False) -> int:
        """Queues the scene (the server takes it over: the Scene object is
        spent afterwards) and returns the job id."""
        o = _abi.FdtdJobOpts(float(end_crit), int(max_timesteps), int(probe_interval), int(keep_fields))
        jid = C.c_uint64()
        check(lib().fdtd_server_submit(self._h, scene._h, C.byref(o), C.byref(jid)), "fdtd_server_submit")
        scene._h = None
        return jid.value

    def status(self, job: int) -> dict:
        st = _abi.FdtdJobStatus()
        check(lib().fdtd_server_job_status(self._h, int(job), C.byref(st)), "fdtd_server_job_status")
        d = {k: getattr(st, k) for k, _ in st._fields_}
        d["num_lines"] = tuple(st.num_lines)
        d["state"] = JOB_STATES[st.state]
        if st.state == 5:
            d["message"] = _abi.last_error()
        return d

    def wait(self, job: int = 0, timeout: float = 0.0):
        """Blocks until the job (0: every submitted job) has finished."""
        check(lib().fdtd_server_wait(self._h, int(job), float(timeout)), "fdtd_server_wait")

    def samples(self, job: int) -> Samples:
        st = self.status(job)
        n, npr = st["num_samples"], st["num_probes"]
        ts = np.zeros(n, np.uint32)
        vals = np.zeros((n, max(npr, 1)), np.float64)
        en = np.zeros(n, np.float64)
        check(lib().fdtd_server_read_samples(self._h, int(job), ts.ctypes.data_as(_abi.PU32),
                                             vals.ctypes.data_as(_abi.PD), en.ctypes.data_as(_abi.PD)),
              "fdtd_server_read_samples")
        types = (C.c_int * max(1, npr))()
        check(lib().fdtd_server_probe_types(self._h, int(job), types, max(1, npr)), "fdtd_server_probe_types")
        return Samples(ts=ts.astype(np.int64), values=vals[:, :npr], energy=en, dT=st["dT"],
                       probe_types=list(types)[:npr])

    def fields(self, job: int):
        shape = (3,) + self.status(job)["num_lines"]
        V = np.empty(shape, np.float32)
        I = np.empty(shape, np.float32)
        check(lib().fdtd_server_get_fields(self._h, int(job), V.ctypes.data_as(_abi.PF), I.ctypes.data_as(_abi.PF)),
              "fdtd_server_get_fields")
        return V, I

    def release(self, job: int):
        check(lib().fdtd_server_release(self._h, int(job)), "fdtd_server_release")

    def stats(self) -> dict:
        st = _abi.FdtdServerStats()
        check(lib().fdtd_server_get_stats(self._h, C.byref(st)), "fdtd_server_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().fdtd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_fdtd(engine: Engine, nr_ts: int, end_crit: float = 1e-6) -> dict:
    """openEMS::RunFDTD's loop: iterate in probe-interval chunks until NrTS
    or until the energy has decayed below end_crit relative to its maximum
    (checked on every sample; the reference checks every ~4 s of wall time,
    openems.cpp:1285-1314)."""
    step = engine.interval or nr_ts
    maxE = 0.0
    change = 1.0
    seen = 0
    while engine.num_timesteps < nr_ts and change > end_crit:
        n = min(step - engine.num_timesteps % step, nr_ts - engine.num_timesteps)
        engine.iterate(n)
        s = engine.samples()
        for e in s.energy[seen:]:
            if e >= 0:
                maxE = max(maxE, e)
                if maxE > 0:
                    change = e / maxE
        seen = len(s.energy)
    return dict(timesteps=engine.num_timesteps, energy_change=change)
