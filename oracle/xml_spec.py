"""ORACLE -- test infrastructure only.

An openEMS XML document (the <FDTD> settings and the CSXCAD
<ContinuousStructure> the front ends write) read into the plain scene
description the oracle's operator build takes (the same dict as
wipems_gb300.SceneSpec.spec), with Python's own XML parser -- a second
reader, independent of the engine library's, restating:

    openEMS::Parse_XML_FDTDSetup     openems.cpp:796-936 (NumberOfTimesteps,
        endCriteria, OverSampling only when > 1, BoundaryCond codes or
        PEC / PMC / MUR / PML_n names, MUR_PhaseVelocity[_face], the
        <Excitation> of Type 0 (Gaussian: f0 fc), 1 (sinusoid: f0), 2 / 3
        (Dirac / step: <FDTD f_max>), 10 (custom: Function, f0))
    default PML size 8               openems.cpp:101
    CSXCAD ContinuousStructure::ReadFromXML, for rectilinear grids
        (DeltaUnit, X/Y/ZLines as sorted unique number lists), the
        background material and the properties Material, LorentzMaterial
        (one order, electric and magnetic families), Metal, LumpedElement (Direction, R, C, L, Caps, LEtype),
        Excitation (Type, Excite, Delay) and ProbeBox (Type, Weight,
        NormDir), each with <Box Priority><P1/><P2/></Box> primitives.

Everything else that changes the simulation raises ValueError; dump boxes
and mode-match probes are skipped (they do not change the fields).
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET

_BNAMES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")


def _num(el, key, default):
    v = el.get(key)
    if v is None:
        return default
    return float(v)


def _nums(text):
    return [float(t) for t in text.replace(";", ",").split(",") if t.strip()]


def _iso(el, key, default):
    """An isotropic material value ("v" or "v,v,v")."""
    if el is None or el.get(key) is None:
        return default
    v = _nums(el.get(key))
    if len(v) == 3 and v[0] == v[1] == v[2]:
        return v[0]
    if len(v) == 1:
        return v[0]
    raise ValueError(f"anisotropic {key}")


def xml_spec(path_or_text: str) -> dict:
    text = path_or_text
    if "<" not in path_or_text:
        with open(path_or_text, encoding="utf-8") as f:
            text = f.read()
    root = ET.fromstring(text)
    if root.tag != "openEMS":
        raise ValueError("root element is not <openEMS>")
    fdtd = root.find("FDTD")
    csx = root.find("ContinuousStructure")
    if fdtd is None or csx is None:
        raise ValueError("<FDTD> and <ContinuousStructure> are required")
    nr = _num(fdtd, "NumberOfTimesteps", 0.0)
    nr_ts = 0 if nr < 0 else int(nr)
    os_ = int(_num(fdtd, "OverSampling", 0))
    oversampling = os_ if os_ > 1 else 4
    if int(_num(fdtd, "CylinderCoords", 0)) == 1:
        raise ValueError("cylindrical coordinates")
    for k in ("TimeStepMethod", "TimeStep", "TimeStepFactor", "MaxTime", "CellConstantMaterial"):
        if fdtd.get(k) is not None:
            raise ValueError(f"<FDTD {k}>")
    exc = fdtd.find("Excitation")
    etype = -1 if exc is None else int(_num(exc, "Type", -1))
    if etype not in (0, 1, 2, 3, 10):
        raise ValueError("only the Gaussian (0), sinusoid (1), Dirac (2), step (3) and custom (10) excitations")
    f0 = _num(exc, "f0", 0.0) if etype in (0, 1, 10) else 0.0
    fc = _num(exc, "fc", 0.0) if etype == 0 else 0.0
    f_max = _num(fdtd, "f_max", 0.0) if etype >= 2 else 0.0
    function = exc.get("Function", "") if etype == 10 else ""
    bcn = fdtd.find("BoundaryCond")
    if bcn is None:
        raise ValueError("<BoundaryCond> missing")
    bc, pml = [0] * 6, [8] * 6  # openEMS's default PML size for every face
    for n, name in enumerate(_BNAMES):
        v = bcn.get(name)
        if v is None:
            continue
        try:
            bc[n] = int(v)  # a bare code keeps the default size
            continue
        except ValueError:
            pass
        if v == "PEC":
            bc[n] = 0
        elif v == "PMC":
            bc[n] = 1
        elif v == "MUR":
            bc[n] = 2
        elif v.startswith("PML_"):
            bc[n] = 3
            digits = ""
            for ch in v[4:]:
                if not ch.isdigit():
                    break
                digits += ch
            pml[n] = int(digits) if digits else 0
    vph = [_num(bcn, "MUR_PhaseVelocity", 0.0)] * 6
    for n, name in enumerate(_BNAMES):
        vph[n] = _num(bcn, "MUR_PhaseVelocity_" + name, vph[n])

    grid = csx.find("RectilinearGrid")
    if grid is None:
        raise ValueError("<RectilinearGrid> missing")
    if int(_num(grid, "CoordSystem", 0)) != 0:
        raise ValueError("cylindrical grid")
    unit = _num(grid, "DeltaUnit", 1.0)
    lines = [sorted(set(_nums(grid.find(t).text))) for t in ("XLines", "YLines", "ZLines")]
    bg = csx.find("BackgroundMaterial")
    background = (1.0, 1.0, 0.0, 0.0)
    if bg is not None:
        background = (_num(bg, "Epsilon", 1.0), _num(bg, "Mue", 1.0), _num(bg, "Kappa", 0.0), _num(bg, "Sigma", 0.0))

    prims = []
    props = csx.find("Properties")
    for p in (list(props) if props is not None else []):
        boxes = []
        pr_el = p.find("Primitives")
        for g in (list(pr_el) if pr_el is not None else []):
            if g.tag != "Box":
                raise ValueError(f"primitive <{g.tag}>")
            if g.find("Transformation") is not None:
                raise ValueError("transformed box")
            a = [_num(g.find("P1"), k, 0.0) for k in "XYZ"]
            b = [_num(g.find("P2"), k, 0.0) for k in "XYZ"]
            boxes.append((int(_num(g, "Priority", 0)), a, b))
        w = p.find("Weight")
        if w is not None and any(float(v) != 1 for v in w.attrib.values()):
            raise ValueError("material weighting functions")
        prop = p.find("Property")
        if p.tag in ("Material", "LorentzMaterial"):
            mat = dict(eps=_iso(prop, "Epsilon", 1.0), mue=_iso(prop, "Mue", 1.0), kappa=_iso(prop, "Kappa", 0.0),
                       sigma=_iso(prop, "Sigma", 0.0))
            if p.tag == "LorentzMaterial":
                if int(_num(p, "Order", 1)) > 1:
                    raise ValueError("dispersion order > 1")
                mat.update(disp_order=1, eps_plasma_f=[_iso(prop, "EpsilonPlasmaFrequency", 0.0)],
                           eps_relax_t=[_iso(prop, "EpsilonRelaxTime", 0.0)],
                           eps_pole_f=[_iso(prop, "EpsilonLorPoleFrequency", 0.0)],
                           mue_plasma_f=[_iso(prop, "MuePlasmaFrequency", 0.0)],
                           mue_relax_t=[_iso(prop, "MueRelaxTime", 0.0)],
                           mue_pole_f=[_iso(prop, "MueLorPoleFrequency", 0.0)])
            for pr, a, b in boxes:
                prims.append(dict(kind="material", priority=pr, start=a, stop=b, **mat))
        elif p.tag == "Metal":
            for pr, a, b in boxes:
                prims.append(dict(kind="metal", priority=pr, start=a, stop=b))
        elif p.tag == "LumpedElement":
            def val(k):
                v = _num(p, k, math.nan)
                return -1.0 if math.isnan(v) else v
            le = dict(ny=int(_num(p, "Direction", -1)), le_type=int(_num(p, "LEtype", 0)), R=val("R"), C=val("C"),
                      L=val("L"), caps=int(_num(p, "Caps", 1) != 0))
            for pr, a, b in boxes:
                prims.append(dict(kind="lumped", priority=pr, start=a, stop=b, **le))
        elif p.tag == "Excitation":
            ex = dict(exc_type=int(_num(p, "Type", 0)), exc_vec=_nums(p.get("Excite")), delay=_num(p, "Delay", 0.0))
            for pr, a, b in boxes:
                prims.append(dict(kind="excitation", priority=pr, start=a, stop=b, **ex))
        elif p.tag == "ProbeBox":
            t = int(_num(p, "Type", 0))
            if t < 0 or t > 3:
                continue
            pb = dict(probe_type=t, weight=_num(p, "Weight", 1.0), norm_dir=int(_num(p, "NormDir", -1)))
            for pr, a, b in boxes:
                prims.append(dict(kind="probe", priority=0, start=a, stop=b, **pb))
        elif p.tag == "DumpBox":
            continue
        else:
            raise ValueError(f"property <{p.tag}>")
    return dict(lines=lines, unit=unit, background=background, bc=bc, pml_size=pml, mur_vph=vph, f0=f0, fc=fc,
                nr_ts=nr_ts, oversampling=oversampling, prims=prims, excite_type=etype, f_max=f_max,
                function=function)
