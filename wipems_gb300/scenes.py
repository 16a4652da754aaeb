"""Seeded synthetic scenes for the benchmark workloads and the parity cases.

No public dataset is involved: every scene is generated from a seed with the
shapes, sizes and value distributions of the workload it stands for.

    p64       64^3 cells, 1 mm, vacuum, PEC, one soft Ez edge, 2000 TS
    l256      256^3 cells, 0.5 mm, UPML-8, 40 dielectric bricks, 50 ohm port, 1000 TS
    d192      192^3 cells, graded 0.2-1 mm, UPML-8, Drude (~25 %) and Lorentz
              (~15 %) bricks, 3000 TS
    b96_job   one job of the 96-job batch (edges 48-160, PEC or UPML-8,
              1-10 bricks, one port, f0 in 1-20 GHz, 1500 TS)
    serve_job one job of the serving stream (edges log-uniform 32-256)
    cavity    the PEC cavity of the reference's resonance test
              (TESTSUITE/combinedtests/cavity.m:37-82)
    drude_metamaterial  the double-negative Drude slab plane wave of the
              reference's example (Metamaterial_PlaneWave_Drude.m)
"""
from __future__ import annotations

import contextlib
import math

import numpy as np

from .fdtd import BC_MUR, BC_PEC, BC_PMC, BC_PML, Scene, SceneSpec

_native = True


@contextlib.contextmanager
def spec_only():
    """Inside this block the generators return SceneSpec objects: the same
    scenes as plain data, built without the engine library (for a checker
    or a CPU baseline that must not load it).  Not thread-safe."""
    global _native
    old = _native
    _native = False
    try:
        yield
    finally:
        _native = old


def _scene(lx, ly, lz, unit):
    return (Scene if _native else SceneSpec)(lx, ly, lz, unit)


def uniform_lines(cells: int, delta: float) -> np.ndarray:
    return np.arange(cells + 1, dtype=np.float64) * delta


def graded_lines(cells: int, rng: np.random.Generator, dmin=0.2, dmax=1.0, ratio=1.3) -> np.ndarray:
    """Seeded graded spacing in [dmin, dmax] with neighbour ratio <= ratio."""
    d = np.empty(cells)
    d[0] = rng.uniform(dmin, dmax)
    lr = math.log(ratio)
    for i in range(1, cells):
        r = math.exp(rng.uniform(-lr, lr))
        d[i] = min(max(d[i - 1] * r, dmin), dmax)
    # snap to a 1e-6 grid so line coordinates are exactly reproducible
    d = np.round(d, 6)
    return np.concatenate([[0.0], np.cumsum(d)]).round(6)


def _pick_box(rng, lines, lo_cell, hi_cell, emin, emax):
    start, stop = [], []
    for a in range(3):
        n = len(lines[a]) - 1
        lo, hi = lo_cell[a], hi_cell[a]
        e = int(rng.integers(emin, min(emax, hi - lo) + 1))
        s = int(rng.integers(lo, hi - e + 1))
        start.append(lines[a][s])
        stop.append(lines[a][s + e])
    return start, stop


def p64(nr_ts: int = 2000) -> Scene:
    """Plain 64^3 PEC vacuum box with one soft Ez edge at the centre."""
    L = uniform_lines(64, 1.0)
    s = _scene(L, L, L, 1e-3)
    s.set_boundary([BC_PEC] * 6)
    s.set_gauss_excite(5e9, 5e9, nr_ts)
    s.add_excitation([32, 32, 32], [32, 32, 33], [0, 0, 1], exc_type=0)
    s.add_probe([42, 32, 22], [42, 32, 42], 0, name="ut_off")
    s.add_probe([31.5, 31.5, 32.5], [32.5, 32.5, 32.5], 1, norm_dir=2, name="it_feed")
    return s


def port_scene(cells, delta, pml, n_bricks, seed, f0, fc, nr_ts, eps_max=12.0, kappa_range=(1e-4, 1.0),
               edge_range=(8, 64), lines=None) -> Scene:
    """Box of dielectric bricks driven by a centred z-directed 50 ohm port."""
    rng = np.random.default_rng(seed)
    if lines is None:
        lines = [uniform_lines(c, delta) for c in cells]
    s = _scene(*lines, 1e-3)
    bc = [BC_PML if pml else BC_PEC] * 6
    s.set_boundary(bc, [pml] * 6 if pml else [0] * 6)
    s.set_gauss_excite(f0, fc, nr_ts)
    lo = [pml + 1 for _ in range(3)]
    hi = [len(lines[a]) - 2 - pml for a in range(3)]
    for b in range(n_bricks):
        emax = min(edge_range[1], min(hi[a] - lo[a] for a in range(3)))
        emin = min(edge_range[0], emax)
        start, stop = _pick_box(rng, lines, lo, hi, emin, emax)
        eps = rng.uniform(1.0, eps_max)
        kappa = math.exp(rng.uniform(math.log(kappa_range[0]), math.log(kappa_range[1]))) if kappa_range else 0.0
        s.add_material(start, stop, eps_r=eps, kappa=kappa, priority=10 + b)
    c = [len(lines[a]) // 2 for a in range(3)]
    start = [lines[0][c[0]], lines[1][c[1]], lines[2][c[2] - 2]]
    stop = [lines[0][c[0] + 1], lines[1][c[1] + 1], lines[2][c[2] + 2]]
    s.add_lumped_port(start, stop, 2, 50.0, excite=1.0, priority=1000)
    return s


def rlc_probe(series: bool, R: float, L: float, Cap: float, nr_ts: int = 8000, cells: int = 24,
              f0: float = 2e9, fc: float = 2e9) -> Scene:
    """One lumped RLC edge (1 mm, z-directed) in a UPML-bounded vacuum box,
    with a voltage probe along the edge and a current loop around it, driven
    by a soft z excitation four cells away.  The loop current is the edge's
    total current (element plus edge capacitance), so V/I is the element's
    impedance in parallel with the edge capacitance."""
    lines = [uniform_lines(cells, 1.0) for _ in range(3)]
    s = _scene(*lines, 1e-3)
    s.set_boundary([BC_PML] * 6, [6] * 6)
    s.set_gauss_excite(f0, fc, nr_ts)
    c = cells // 2
    a = [lines[0][c], lines[1][c], lines[2][c]]
    b = [lines[0][c], lines[1][c], lines[2][c + 1]]
    s.add_lumped_rlc(a, b, 2, R=R, L=L, Cap=Cap, series=series, caps=False, priority=10)
    s.add_excitation([lines[0][c - 4], lines[1][c], lines[2][c]], [lines[0][c - 4], lines[1][c], lines[2][c + 1]],
                     [0.0, 0.0, 1.0], priority=10)
    s.add_probe(a, b, 0, name="v")
    half = 0.5 * (lines[2][c] + lines[2][c + 1])
    s.add_probe([lines[0][c] - 0.5, lines[1][c] - 0.5, half], [lines[0][c] + 0.5, lines[1][c] + 0.5, half], 1,
                norm_dir=2, name="i")
    return s


def l256(nr_ts: int = 1000, seed: int = 256, cells: int = 256, n_bricks: int = 40) -> Scene:
    """256^3 cells at 0.5 mm, UPML-8, 40 bricks (edge 8-64 cells, eps_r
    U[1,12], kappa log-U[1e-4,1] S/m), 50 ohm z port with a Gaussian pulse."""
    return port_scene([cells] * 3, 0.5, 8, n_bricks, seed, 10e9, 10e9, nr_ts, edge_range=(8, 64))


def d192(nr_ts: int = 3000, seed: int = 192, cells: int = 192, pml: int = 8) -> Scene:
    """192^3 graded cells, UPML-8, Drude (~25 % of cells) and single-pole
    Lorentz (~15 %) bricks.  Frequencies are the optical values scaled by the
    nm -> mm geometry factor 1e-6 so the pulse and the media interact on
    this mesh: Drude f_p = 2e15*1e-6 Hz, collision 1e13..1e14 /s * 1e-6."""
    rng = np.random.default_rng(seed)
    lines = [graded_lines(cells, rng) for _ in range(3)]
    s = _scene(*lines, 1e-3)
    s.set_boundary([BC_PML] * 6, [pml] * 6)
    s.set_gauss_excite(6e9, 6e9, nr_ts)
    lo = [pml + 1] * 3
    hi = [cells - 1 - pml] * 3
    occ_d = np.zeros((cells,) * 3, bool)
    occ_l = np.zeros((cells,) * 3, bool)
    prio = 10
    scale = 1e-6
    tries = 0
    while (occ_d.mean() < 0.25 or occ_l.mean() < 0.15) and tries < 400:
        tries += 1
        drude = occ_d.mean() < 0.25 and (occ_l.mean() >= 0.15 or rng.random() < 0.6)
        emin, emax = 12, 48
        idx0, idx1 = [], []
        for a in range(3):
            e = int(rng.integers(emin, emax + 1))
            st = int(rng.integers(lo[a], hi[a] - e + 1))
            idx0.append(st)
            idx1.append(st + e)
        start = [lines[a][idx0[a]] for a in range(3)]
        stop = [lines[a][idx1[a]] for a in range(3)]
        sl = tuple(slice(idx0[a], idx1[a]) for a in range(3))
        if drude:
            nu = math.exp(rng.uniform(math.log(1e13), math.log(1e14))) * scale
            s.add_lorentz(start, stop, eps_r=1.0, plasma_f=[2e15 * scale], relax_t=[1.0 / nu], pole_f=[0.0],
                          priority=prio)
            occ_d[sl] = True
            occ_l[sl] = False
        else:
            eps_inf = rng.uniform(2, 4)
            deps = rng.uniform(1, 5)
            fL = rng.uniform(2e9, 20e9)
            nu = math.exp(rng.uniform(math.log(1e8), math.log(1e9)))
            s.add_lorentz(start, stop, eps_r=eps_inf, plasma_f=[fL * math.sqrt(deps)], relax_t=[1.0 / nu],
                          pole_f=[fL], priority=prio)
            occ_l[sl] = True
            occ_d[sl] = False
        prio += 1
    c = [cells // 2] * 3
    start = [lines[0][c[0]], lines[1][c[1]], lines[2][c[2] - 2]]
    stop = [lines[0][c[0] + 1], lines[1][c[1] + 1], lines[2][c[2] + 2]]
    s.add_lumped_port(start, stop, 2, 50.0, excite=1.0, priority=10000)
    s.meta = dict(drude_fraction=float(occ_d.mean()), lorentz_fraction=float(occ_l.mean()))
    return s


def b96_job(seed: int, nr_ts: int = 1500) -> Scene:
    """One job of the 96-job sweep."""
    rng = np.random.default_rng(10_000 + seed)
    cells = [int(rng.integers(48, 161)) for _ in range(3)]
    pml = 8 if seed % 2 else 0
    n_bricks = int(rng.integers(1, 11))
    f0 = float(rng.uniform(1e9, 20e9))
    return port_scene(cells, 0.5, pml, n_bricks, 20_000 + seed, f0, f0 / 2, nr_ts, eps_max=10.0, kappa_range=None,
                      edge_range=(4, 32))


def serve_job(seed: int, nr_ts: int = 20000) -> Scene:
    """One request of the serving stream: edges log-uniform in [32, 256]
    cells, 60 % dielectric + UPML, 40 % Drude or Lorentz bricks."""
    rng = np.random.default_rng(30_000 + seed)
    cells = [int(round(math.exp(rng.uniform(math.log(32), math.log(256))))) for _ in range(3)]
    kind = "dielectric" if rng.random() < 0.6 else ("drude" if rng.random() < 0.5 else "lorentz")
    f0 = float(rng.uniform(2e9, 15e9))
    lines = [uniform_lines(c, 0.5) for c in cells]
    if kind == "dielectric":
        s = port_scene(cells, 0.5, 8, int(rng.integers(1, 8)), 40_000 + seed, f0, f0 / 2, nr_ts, eps_max=10.0,
                       kappa_range=None, edge_range=(4, 24), lines=lines)
    else:
        s = _scene(*lines, 1e-3)
        s.set_boundary([BC_PML] * 6, [8] * 6)
        s.set_gauss_excite(f0, f0 / 2, nr_ts)
        for b in range(int(rng.integers(1, 6))):
            lo = [9] * 3
            hi = [c - 9 for c in cells]
            emax = max(2, min(24, min(hi[a] - lo[a] for a in range(3))))
            start, stop = _pick_box(rng, lines, lo, hi, min(4, emax), emax)
            if kind == "drude":
                nu = math.exp(rng.uniform(math.log(1e7), math.log(1e8)))
                s.add_lorentz(start, stop, plasma_f=[2e9], relax_t=[1.0 / nu], pole_f=[0.0], priority=10 + b)
            else:
                fL = rng.uniform(2e9, 20e9)
                s.add_lorentz(start, stop, eps_r=rng.uniform(2, 4), plasma_f=[fL * math.sqrt(rng.uniform(1, 5))],
                              relax_t=[1e-9], pole_f=[fL], priority=10 + b)
        c = [n // 2 for n in cells]
        start = [lines[0][c[0]], lines[1][c[1]], lines[2][c[2] - 2]]
        stop = [lines[0][c[0] + 1], lines[1][c[1] + 1], lines[2][c[2] + 2]]
        s.add_lumped_port(start, stop, 2, 50.0, excite=1.0, priority=1000)
    s.meta = dict(kind=kind, cells=cells)
    return s


def cavity(nr_ts: int = 20000) -> Scene:
    """PEC cavity a x b x d = 50 x 20 x 60 mm of the reference's resonance
    test (TESTSUITE/combinedtests/cavity.m:37-117): mesh linspace(0,a,26) x
    linspace(0,b,11) x linspace(0,d,32), Gaussian f0 = fc = 4.5 GHz, a
    one-cell staircase excitation in [1 1 1] near 2/3 of the box, voltage
    probes ut1x/ut1y/ut1z."""
    a, b, d = 50.0, 20.0, 60.0
    mx = np.linspace(0, a, 26)
    my = np.linspace(0, b, 11)
    mz = np.linspace(0, d, 32)
    s = _scene(mx, my, mz, 1e-3)
    s.set_boundary([BC_PEC] * 6)
    f_start, f_stop = 1e9, 10e9
    s.set_gauss_excite((f_stop - f_start) / 2, (f_stop - f_start) / 2, nr_ts)
    i, j, k = int(26 * 2 / 3) - 1, int(11 * 2 / 3) - 1, int(32 * 2 / 3) - 1
    # staircase x-edge, y-edge, z-edge from node (i,j,k) to (i+1,j+1,k+1)
    s.add_excitation([mx[i], my[j], mz[k]], [mx[i + 1], my[j], mz[k]], [1, 1, 1], priority=1)
    s.add_excitation([mx[i + 1], my[j], mz[k]], [mx[i + 1], my[j + 1], mz[k]], [1, 1, 1], priority=2)
    s.add_excitation([mx[i + 1], my[j + 1], mz[k]], [mx[i + 1], my[j + 1], mz[k + 1]], [1, 1, 1], priority=3)
    xi, yi, zi = int(26 / 4) - 1, int(11 / 2) - 1, int(32 / 5) - 1
    s.add_probe([mx[xi], my[yi], mz[zi]], [mx[xi + 1], my[yi], mz[zi]], 0, name="ut1x")
    s.add_probe([mx[xi], my[yi], mz[zi]], [mx[xi], my[yi + 1], mz[zi]], 0, name="ut1y")
    xm = int(26 / 2) - 1
    s.add_probe([mx[xm], my[yi], mz[zi]], [mx[xm], my[yi], mz[zi + 1]], 0, name="ut1z")
    s.meta = dict(a=a * 1e-3, b=b * 1e-3, d=d * 1e-3, f_start=f_start, f_stop=f_stop)
    return s


def mini(kind: str, seed: int = 0, nr_ts: int = 400) -> Scene:
    """Small scenes exercising each feature of the big workloads (parity
    cases the CPU oracle finishes in seconds); odd sizes hit tile edges."""
    if kind == "pec":
        return port_scene([21, 17, 37], 1.0, 0, 3, seed, 5e9, 5e9, nr_ts, edge_range=(2, 6))
    if kind == "upml":
        return port_scene([33, 29, 41], 0.5, 6, 5, seed, 10e9, 10e9, nr_ts, edge_range=(2, 8))
    if kind == "mur":  # Mur on five faces, PEC below, dielectric bricks, lumped port
        s = port_scene([31, 27, 39], 0.5, 0, 4, seed, 10e9, 10e9, nr_ts, edge_range=(2, 8))
        s.set_boundary([BC_MUR, BC_MUR, BC_MUR, BC_MUR, BC_PEC, BC_MUR], [0] * 6)
        return s
    if kind in ("rlc", "rlc_mur"):  # series and parallel lumped RLC elements beside the port
        cells = [33, 29, 41]
        s = port_scene(cells, 0.5, 6 if kind == "rlc" else 0, 3, seed, 10e9, 10e9, nr_ts, edge_range=(2, 8))
        lines = [uniform_lines(n, 0.5) for n in cells]
        c = [n // 2 for n in cells]
        # series R-L-C along z over three cells, one edge wide
        s.add_lumped_rlc([lines[0][c[0] - 4], lines[1][c[1]], lines[2][c[2] - 2]],
                         [lines[0][c[0] - 4], lines[1][c[1]], lines[2][c[2] + 1]], 2,
                         R=20.0, L=1e-9, Cap=0.5e-12, series=True, caps=False, priority=900)
        # parallel R || L || C along x over two cells, two lines across, with caps
        s.add_lumped_rlc([lines[0][c[0] + 3], lines[1][c[1] - 1], lines[2][c[2]]],
                         [lines[0][c[0] + 5], lines[1][c[1]], lines[2][c[2]]], 0,
                         R=200.0, L=3e-9, Cap=0.2e-12, caps=True, priority=900)
        if kind == "rlc_mur":
            s.set_boundary([BC_MUR, BC_MUR, BC_MUR, BC_MUR, BC_PEC, BC_MUR], [0] * 6)
            # a series element on the xmin Mur face line (the face's apply overwrites it)
            s.add_lumped_rlc([lines[0][0], lines[1][c[1] + 3], lines[2][c[2] - 2]],
                             [lines[0][0], lines[1][c[1] + 3], lines[2][c[2]]], 2,
                             R=50.0, L=2e-9, Cap=1e-12, series=True, caps=False, priority=900)
        return s
    if kind == "graded":
        rng = np.random.default_rng(seed)
        lines = [graded_lines(c, rng) for c in (30, 26, 35)]
        return port_scene([30, 26, 35], None, 4, 4, seed, 8e9, 8e9, nr_ts, edge_range=(2, 8), lines=lines)
    if kind in ("drude", "lorentz", "mixed"):
        rng = np.random.default_rng(seed)
        cells = [34, 30, 38]
        lines = [graded_lines(c, rng) for c in cells] if kind == "mixed" else [uniform_lines(c, 0.5) for c in cells]
        s = _scene(*lines, 1e-3)
        s.set_boundary([BC_PML] * 6, [5] * 6)
        s.set_gauss_excite(8e9, 8e9, nr_ts)
        for b in range(4):
            start, stop = _pick_box(rng, lines, [6] * 3, [c - 6 for c in cells], 3, 10)
            use_lor = (kind == "lorentz") or (kind == "mixed" and b % 2)
            if use_lor:
                fL = rng.uniform(4e9, 20e9)
                s.add_lorentz(start, stop, eps_r=rng.uniform(2, 4), plasma_f=[fL * math.sqrt(rng.uniform(1, 5))],
                              relax_t=[1e-9], pole_f=[fL], priority=10 + b)
            else:
                s.add_lorentz(start, stop, plasma_f=[2e9], relax_t=[1.0 / rng.uniform(1e7, 1e8)], pole_f=[0.0],
                              priority=10 + b)
        c = [n // 2 for n in cells]
        start = [lines[0][c[0]], lines[1][c[1]], lines[2][c[2] - 2]]
        stop = [lines[0][c[0] + 1], lines[1][c[1] + 1], lines[2][c[2] + 2]]
        s.add_lumped_port(start, stop, 2, 50.0, excite=1.0, priority=1000)
        return s
    if kind in ("multipole", "multipole_graded"):
        # Lorentz/Drude materials of dispersion order 2 and 3 (several poles
        # per material, as metal models use): a Drude pole plus two Lorentz
        # poles, a Lorentz pole plus a Drude pole with a magnetic second
        # order, and an order-2 material beside an order-1 one
        rng = np.random.default_rng(seed)
        cells = [34, 30, 38]
        graded = kind == "multipole_graded"
        lines = [graded_lines(c, rng) for c in cells] if graded else [uniform_lines(c, 0.5) for c in cells]
        s = _scene(*lines, 1e-3)
        s.set_boundary([BC_PML] * 6, [5] * 6)
        s.set_gauss_excite(8e9, 8e9, nr_ts)
        boxes = [_pick_box(rng, lines, [6] * 3, [c - 6 for c in cells], 3, 10) for _ in range(3)]
        s.add_lorentz(*boxes[0], eps_r=2.0, plasma_f=[6e9, 9e9, 4e9], relax_t=[1e-9, 2e-9, 0.5e-9],
                      pole_f=[0.0, 7e9, 11e9], priority=10)
        s.add_lorentz(*boxes[1], eps_r=3.0, plasma_f=[5e9, 8e9], relax_t=[1e-9, 1e-9], pole_f=[6e9, 0.0],
                      mue_plasma_f=[0.0, 4e9], mue_relax_t=[0.0, 1e-9], priority=11)
        s.add_lorentz(*boxes[2], eps_r=1.5, plasma_f=[3e9], relax_t=[2e-9], priority=12)
        c = [n // 2 for n in cells]
        start = [lines[0][c[0]], lines[1][c[1]], lines[2][c[2] - 2]]
        stop = [lines[0][c[0] + 1], lines[1][c[1] + 1], lines[2][c[2] + 2]]
        s.add_lumped_port(start, stop, 2, 50.0, excite=1.0, priority=1000)
        return s
    if kind in ("magnetic", "magnetic_graded"):
        # the magnetic (mue) family of the Lorentz material, alone and with
        # the electric one: a double-negative Drude box, a magnetic Lorentz
        # pole, an electric Lorentz pole with a magnetic Drude term, and a
        # magnetic-only Drude box
        rng = np.random.default_rng(seed)
        cells = [34, 30, 38]
        graded = kind == "magnetic_graded"
        lines = [graded_lines(c, rng) for c in cells] if graded else [uniform_lines(c, 0.5) for c in cells]
        s = _scene(*lines, 1e-3)
        s.set_boundary([BC_PML] * 6, [5] * 6)
        s.set_gauss_excite(8e9, 8e9, nr_ts)
        for b in range(4):
            start, stop = _pick_box(rng, lines, [6] * 3, [c - 6 for c in cells], 3, 10)
            fp = rng.uniform(3e9, 9e9)
            tau = 1.0 / rng.uniform(1e8, 1e9)
            if b == 0:
                s.add_lorentz(start, stop, plasma_f=[fp], relax_t=[tau], mue_plasma_f=[fp], mue_relax_t=[tau],
                              priority=10 + b)
            elif b == 1:
                fL = rng.uniform(4e9, 12e9)
                s.add_lorentz(start, stop, mue_r=rng.uniform(1, 3), mue_plasma_f=[fL * math.sqrt(rng.uniform(1, 4))],
                              mue_relax_t=[1e-9], mue_pole_f=[fL], priority=10 + b)
            elif b == 2:
                fL = rng.uniform(4e9, 12e9)
                s.add_lorentz(start, stop, eps_r=rng.uniform(2, 4), plasma_f=[fL * math.sqrt(rng.uniform(1, 4))],
                              relax_t=[1e-9], pole_f=[fL], mue_plasma_f=[fp], mue_relax_t=[tau], priority=10 + b)
            else:
                s.add_lorentz(start, stop, mue_plasma_f=[fp], mue_relax_t=[tau], priority=10 + b)
        c = [n // 2 for n in cells]
        start = [lines[0][c[0]], lines[1][c[1]], lines[2][c[2] - 2]]
        stop = [lines[0][c[0] + 1], lines[1][c[1] + 1], lines[2][c[2] + 2]]
        s.add_lumped_port(start, stop, 2, 50.0, excite=1.0, priority=1000)
        h = [lines[0][c[0] - 3], lines[1][c[1] + 2], lines[2][c[2]]]
        s.add_probe(h, h, 3, name="H")
        return s
    raise ValueError(kind)


def drude_metamaterial(nr_ts: int = 6000, length_mm: float = 500.0) -> Scene:
    """A quasi-2D plane wave through a double-negative Drude slab: the
    configuration of the reference's example
    (matlab/examples/other/Metamaterial_PlaneWave_Drude.m:21-80): a 10 x 1.5
    x length mm channel at 0.5 mm, PMC on x, PEC on y, Mur on z, a Gaussian
    of f0 = 0 and fc = 10 GHz with oversampling 10, E_y excited on the third
    z line, and a slab over the middle half of z whose eps and mue both
    follow a Drude model of plasma frequency 5 GHz and relaxation time 5 ns.
    Voltage probes (E_y across the channel) before, in and behind the slab."""
    res = 0.5
    mx = np.arange(-5.0, 5.0 + res / 2, res)
    my = np.arange(-0.75, 0.75 + res / 2, res)
    mz = np.arange(-length_mm / 2, length_mm / 2 + res / 2, res)
    s = _scene(mx, my, mz, 1e-3)
    s.set_boundary([BC_PMC, BC_PMC, BC_PEC, BC_PEC, BC_MUR, BC_MUR], [0] * 6)
    s.set_gauss_excite(0.0, 10e9, nr_ts)
    s.set_oversampling(10)
    s.add_excitation([mx[0], my[0], mz[2]], [mx[-1], my[-1], mz[2]], [0, 1, 0], priority=0)
    f0, tau = 5e9, 5e-9
    s.add_lorentz([mx[0], my[0], -length_mm / 4], [mx[-1], my[-1], length_mm / 4], eps_r=1.0, mue_r=1.0,
                  plasma_f=[f0], relax_t=[tau], mue_plasma_f=[f0], mue_relax_t=[tau], priority=10)
    for name, zc in (("before", -length_mm * 0.375), ("inside", 0.0), ("behind", length_mm * 0.375)):
        k = int(np.argmin(np.abs(mz - zc)))
        s.add_probe([0.0, my[0], mz[k]], [0.0, my[-1], mz[k]], 0, name=name)
    s.meta = dict(f0=f0, relax_t=tau)
    return s
