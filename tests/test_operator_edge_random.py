"""Seeded hostile scenes for the two operator builds: boxes reaching out of
the grid or lying wholly outside it, corners given in either order,
zero-thickness sheets and single lines, primitives tied on priority (the
first added wins), extreme material values (large epsilon, kappa and sigma,
metal-like conductors), lumped R / RLC elements anywhere, probes outside
the grid or degenerate, excitations
with zero components and delays.  The product's operator build
and the oracle's independent one must agree on every array, dT and every
snapped probe, or both refuse the scene; non-finite coefficients appear
only where openEMS has them too, and the compressor refuses those.  CPU
only."""
import math

import numpy as np
import pytest

import oracle
from wipems_gb300 import CompressedOperator, Operator, Scene
from wipems_gb300._abi import FdtdError
from wipems_gb300.fdtd import BC_MUR, BC_PEC, BC_PMC, BC_PML
from wipems_gb300.scenes import graded_lines, uniform_lines

from helpers import assert_same_operator

pytestmark = pytest.mark.usefixtures("libs")


def _coord(rng, ln, margin=3):
    """A coordinate on a line, between lines, or beyond the grid."""
    r = rng.random()
    lo, hi = float(ln[0]), float(ln[-1])
    if r < 0.55:
        return float(ln[int(rng.integers(0, len(ln)))])
    if r < 0.85:
        k = int(rng.integers(0, len(ln) - 1))
        return float(ln[k] + rng.uniform(0.05, 0.95) * (ln[k + 1] - ln[k]))
    span = hi - lo
    return float(rng.choice([lo - rng.uniform(0.1, 0.3) * span, hi + rng.uniform(0.1, 0.3) * span]))


def _box(rng, lines):
    a = [_coord(rng, ln) for ln in lines]
    b = [_coord(rng, ln) for ln in lines]
    for k in range(3):
        r = rng.random()
        if r < 0.15:
            b[k] = a[k]            # a sheet (or a line, or a point)
    return a, b


def hostile_scene(seed: int) -> Scene:
    rng = np.random.default_rng(seed)
    cells = [int(rng.integers(4, 26)) for _ in range(3)]
    if rng.random() < 0.3:
        lines = [graded_lines(c, rng) for c in cells]
    else:
        lines = [uniform_lines(c, float(rng.choice([0.25, 1.0]))) for c in cells]
    s = Scene(*lines, 1e-3)
    bc = [int(rng.choice([BC_PEC, BC_PMC, BC_MUR, BC_PML])) for _ in range(6)]
    pml = [int(rng.integers(1, 6)) if b == BC_PML else 0 for b in bc]
    s.set_boundary(bc, pml)
    if rng.random() < 0.3:
        s.set_background(eps_r=float(rng.uniform(1, 4)), kappa=float(rng.uniform(0, 1e-3)))
    f0 = float(rng.uniform(1e9, 30e9))
    s.set_gauss_excite(f0, f0 * float(rng.uniform(0.3, 1.0)), 100)
    prio = lambda: int(rng.integers(-3, 4))  # noqa: E731  (ties on purpose)
    for _ in range(int(rng.integers(1, 9))):
        a, b = _box(rng, lines)
        r = rng.random()
        if r < 0.2:
            s.add_metal(a, b, priority=prio())
        elif r < 0.35:
            s.add_material(a, b, eps_r=float(rng.choice([1.0, 80.0, 1e4])), kappa=float(rng.choice([0.0, 1e3, 5e7])),
                           mue_r=float(rng.choice([1.0, 50.0])), sigma=float(rng.choice([0.0, 1e4])), priority=prio())
        elif r < 0.5:
            fp = float(rng.uniform(1e9, 2e10))
            s.add_lorentz(a, b, eps_r=float(rng.uniform(1, 5)), plasma_f=[fp], relax_t=[float(rng.uniform(1e-11, 1e-8))],
                          pole_f=[float(rng.choice([0.0, fp / 2]))], priority=prio())
        else:
            s.add_material(a, b, eps_r=float(rng.uniform(1, 12)), kappa=float(rng.uniform(0, 1.0)), priority=prio())
    for _ in range(int(rng.integers(1, 3))):
        a, b = _box(rng, lines)
        vec = [float(rng.choice([0.0, -1.0, 2.5])) for _ in range(3)]
        s.add_excitation(a, b, vec, delay=float(rng.choice([0.0, 1e-10, 3.7e-11])), priority=prio())
    for _ in range(int(rng.integers(0, 3))):
        a, b = _box(rng, lines)
        d = int(rng.integers(0, 3))
        r = rng.random()
        if r < 0.4:
            s.add_lumped(a, b, d, R=float(rng.choice([50.0, 0.0, 1e6])), Cap=float(rng.choice([-1.0, 1e-12])),
                         caps=bool(rng.random() < 0.5), priority=prio())
        else:
            s.add_lumped_rlc(a, b, d, R=float(rng.choice([-1.0, 10.0, 300.0])), L=float(rng.choice([-1.0, 1e-9])),
                             Cap=float(rng.choice([-1.0, 1e-12])), series=bool(rng.random() < 0.5),
                             caps=bool(rng.random() < 0.5), priority=prio())
    for _ in range(int(rng.integers(0, 5))):
        a, b = _box(rng, lines)
        s.add_probe(a, b, int(rng.integers(0, 4)), weight=float(rng.choice([1.0, -1.0, 0.5])),
                    norm_dir=int(rng.integers(-1, 3)))
    return s


def _build(make):
    try:
        return make(), None
    except FdtdError as ex:
        return None, ex
    except (RuntimeError, ValueError) as ex:
        return None, ex


@pytest.mark.parametrize("seed", range(150))
def test_hostile_scenes_build_identically(seed):
    scene = hostile_scene(seed)
    prod, perr = _build(lambda: Operator(scene))
    ref, rerr = _build(lambda: oracle.Operator(scene.spec))
    assert (prod is None) == (ref is None), (perr, rerr)
    if prod is None:
        return
    assert_same_operator(prod, ref)
    assert math.isfinite(prod.dT) and prod.dT > 0
    # openEMS turns an unset lumped R, L or C into NaN, so an under-specified
    # RLC element has NaN coefficients in both builds (as in openEMS); the
    # compressor refuses such an operator rather than run it.  Any other
    # non-finite coefficient is an error.
    arrs = oracle.desc_arrays(prod.desc)
    bad = [k for k, v in arrs.items() if v.dtype.kind == "f" and not np.all(np.isfinite(v))]
    assert all(k.startswith("rlc.") for k in bad), bad
    if bad:  # refused (by this check, or by an earlier one)
        with pytest.raises(FdtdError):
            CompressedOperator(prod)


@pytest.mark.parametrize("seed", range(0, 150, 3))
def test_hostile_scenes_as_xml_read_identically(seed):
    """The hostile scenes written as openEMS XML documents (random spellings,
    as in test_xml_random.py): the engine library's reader + operator build
    and the oracle's reader + operator build agree, or both refuse."""
    from oracle.xml_spec import xml_spec
    from test_xml_random import spec_xml
    text = spec_xml(hostile_scene(seed).spec, np.random.default_rng(9000 + seed))
    prod, perr = _build(lambda: Operator(Scene.from_xml(text)))
    ref, rerr = _build(lambda: oracle.Operator(xml_spec(text)))
    assert (prod is None) == (ref is None), (perr, rerr)
    if prod is not None:
        assert_same_operator(prod, ref)


@pytest.mark.parametrize("seed", range(40))
def test_scene_api_survives_bad_values(seed):
    """NaN, infinite, negative and huge values in the scene calls: every
    call either takes the value or refuses it with a status, and the
    operator build and compression end in a result or a status, never in a
    crash (a crash here ends the test process)."""
    rng = np.random.default_rng(11000 + seed)
    bad = [float("nan"), float("inf"), -float("inf"), -1.0, 0.0, 1e300, -1e300, 1e-300]

    def v():
        return float(rng.choice(bad)) if rng.random() < 0.08 else float(rng.uniform(0, 10))

    lines = [np.arange(0, 10.5, 0.5)] * 3
    s = Scene(*lines, 1e-3)
    try:
        s.set_boundary([int(rng.choice([0, 1, 2, 3, 3, 3])) for _ in range(6)],
                       [int(rng.choice([0, 2, 8, 3, 1])) for _ in range(6)])
    except FdtdError:
        return
    for _ in range(6):
        k = int(rng.integers(0, 6))
        a, b = [v() for _ in range(3)], [v() for _ in range(3)]
        try:
            if k == 0:
                s.add_material(a, b, eps_r=v(), kappa=v(), mue_r=v(), sigma=v(), priority=int(rng.integers(-5, 5)))
            elif k == 1:
                s.add_metal(a, b)
            elif k == 2:
                s.add_excitation(a, b, [v(), v(), v()], delay=v())
            elif k == 3:
                s.add_probe(a, b, int(rng.integers(-1, 5)), weight=v(), norm_dir=int(rng.integers(-2, 4)))
            elif k == 4:
                s.add_lumped(a, b, int(rng.integers(-1, 4)), R=v(), Cap=v())
            else:
                s.add_lorentz(a, b, eps_r=v(), plasma_f=[v()], relax_t=[v()], pole_f=[v()])
        except FdtdError:
            pass
    try:
        s.set_gauss_excite(v(), v(), int(rng.integers(1, 50)))
    except FdtdError:
        pass
    try:
        CompressedOperator(Operator(s))
    except FdtdError:
        pass
