"""Shared helpers of the test suite (comparison metrics and the frequency
check of the reference's TESTSUITE)."""
from __future__ import annotations

import numpy as np


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b)
    if n == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / n)


def rel_max(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m = np.max(np.abs(b))
    if m == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / m)


def fft_time2freq(t, val):
    """matlab/FFT_time2freq.m: zero-padded single-sided spectrum."""
    dt = t[1] - t[0]
    L = len(t)
    nfft = 1 << int(np.ceil(np.log2(L)))
    v = np.fft.fft(val, nfft) * dt
    f = 1 / (2 * dt) * np.linspace(0, 1, nfft // 2 + 1)
    v = 2 * v[: nfft // 2 + 1]
    return f, v


def _nearest(f, x):
    return int(np.argmin(np.abs(f - x)))


def check_frequency(f, val, f_upper, f_lower, rel_amplitude, kind) -> bool:
    """TESTSUITE/helperscripts/check_frequency.m."""
    max1 = np.max(val)
    for f1, f2 in zip(f_lower, f_upper):
        i1, i2 = _nearest(f, f1), _nearest(f, f2)
        seg = val[i1:i2 + 1]
        if kind == "inside" and np.max(seg) < max1 * rel_amplitude:
            return False
        if kind == "outside" and np.max(seg) > max1 * rel_amplitude:
            return False
    return True


def cavity_check(t_list, val_list, meta) -> dict:
    """Analysis of TESTSUITE/combinedtests/cavity.m:125-214 on the probes
    ut1x, ut1y, ut1z (time series); returns the four pass flags."""
    c0 = 299792458.0
    a, b, d = meta["a"], meta["b"], meta["d"]
    f_start, f_stop = meta["f_start"], meta["f_stop"]
    t_start = 7e-10
    spec = []
    for t, v in zip(t_list, val_list):
        i0 = _nearest(t, t_start)
        f, s = fft_time2freq(t[i0:], v[i0:])
        spec.append((f, s))
    f = spec[0][0]
    i1, i2 = _nearest(f, f_start), _nearest(f, f_stop)
    f = f[i1:i2 + 1]
    uy = np.abs(spec[1][1][i1:i2 + 1])
    uz = np.abs(spec[2][1][i1:i2 + 1])
    k = lambda m, n, l: np.sqrt((m * np.pi / a) ** 2 + (n * np.pi / b) ** 2 + (l * np.pi / d) ** 2)
    f_TE = np.array([c0 / (2 * np.pi) * k(*m) for m in [(1, 0, 1), (1, 0, 2), (2, 0, 1), (2, 0, 2)]])
    f_TM = np.array([c0 / (2 * np.pi) * k(*m) for m in [(1, 1, 0), (1, 1, 1)]])
    lower, upper, lower_TM, upper_TM = 1.3e-3, 1.3e-3, 2.5e-3, 0.0
    min_amp, min_amp_TM, outer, max_amp = 0.6, 0.27, 0.02, 0.17

    def outer_lims(fr):
        temp = np.concatenate([[f_start], fr, [f_stop]])
        o1 = temp[:-1] * (1 + outer)
        o2 = temp[1:] * (1 - outer)
        return o1, o2

    o1, o2 = outer_lims(f_TE)
    o1t, o2t = outer_lims(f_TM)
    return dict(
        te_inside=check_frequency(f, uy, f_TE * (1 + upper), f_TE * (1 - lower), min_amp, "inside"),
        tm_inside=check_frequency(f, uz, f_TM * (1 + upper_TM), f_TM * (1 - lower_TM), min_amp_TM, "inside"),
        te_outside=check_frequency(f, uy, o2, o1, max_amp, "outside"),
        tm_outside=check_frequency(f, uz, o2t, o1t, max_amp, "outside"),
    )


def edge_lengths(lines, unit, dual):
    """Operator::GetEdgeLength along one axis (GetDiscDelta * grid delta)."""
    l = np.asarray(lines, np.float64)
    n = len(l)
    dl = np.empty(n)
    if not dual:
        dl[:-1] = l[1:] - l[:-1]
        dl[-1] = l[-1] - l[-2]
    else:
        d = np.empty(n)  # dual lines
        d[:-1] = 0.5 * (l[:-1] + l[1:])
        d[-1] = l[-1] + 0.5 * (l[-1] - l[-2])
        dl[1:] = d[1:] - d[:-1]
        dl[0] = l[1] - l[0]
    return dl * unit


def dump_reference(V, I, lines, unit, field, interp, start, stop, step):
    """Engine_Interface_FDTD::GetRawInterpolated(Dual)Field at the dump lines
    (engine_interface_fdtd.cpp:60-200), point by point in the reference's
    order, double arithmetic, stored as float (processfields.cpp:280-330)."""
    N = V.shape[1:]
    Lm = [edge_lengths(lines[a], unit, False) for a in range(3)]
    Ld = [edge_lengths(lines[a], unit, True) for a in range(3)]
    idx = [list(range(min(start[a], stop[a]), max(start[a], stop[a]) + 1, max(1, step[a]))) for a in range(3)]
    out = np.zeros((3, len(idx[0]), len(idx[1]), len(idx[2])), np.float32)

    def rawE(n, p):
        d = Lm[n][p[n]]
        return float(V[n][p[0], p[1], p[2]]) / d if d != 0 else 0.0

    def rawH(n, p):
        d = Ld[n][p[n]]
        return float(I[n][p[0], p[1], p[2]]) / d if d != 0 else 0.0

    for i, x in enumerate(idx[0]):
        for j, y in enumerate(idx[1]):
            for k, z in enumerate(idx[2]):
                p = [x, y, z]
                top = any(p[a] == N[a] - 1 for a in range(3))
                for n in range(3):
                    nP, nPP = (n + 1) % 3, (n + 2) % 3
                    q = list(p)
                    if field == "E":
                        if interp == "none":
                            o = rawE(n, p)
                        elif interp == "node":
                            if p[n] == N[n] - 1:
                                q[n] -= 1
                                o = rawE(n, q)
                            elif Lm[n][p[n]] == 0:
                                o = 0.0
                            elif p[n] == 0:
                                o = rawE(n, p)
                            else:
                                delta = Lm[n][p[n]]
                                q[n] -= 1
                                rel = delta / (delta + Lm[n][q[n]])
                                o = rawE(n, p) * (1.0 - rel) + rawE(n, q) * rel
                        else:
                            if top:
                                o = 0.0
                            else:
                                o = rawE(n, q)
                                q[nP] += 1
                                o += rawE(n, q)
                                q[nPP] += 1
                                o += rawE(n, q)
                                q[nP] -= 1
                                o += rawE(n, q)
                                o /= 4
                    else:
                        if interp == "none":
                            o = rawH(n, p)
                        elif interp == "node":
                            if top or p[nP] == 0 or p[nPP] == 0:
                                o = 0.0
                            else:
                                o = rawH(n, q)
                                q[nP] -= 1
                                o += rawH(n, q)
                                q[nPP] -= 1
                                o += rawH(n, q)
                                q[nP] += 1
                                o += rawH(n, q)
                                o /= 4
                        else:
                            if p[n] >= N[n] - 1:
                                o = 0.0
                            else:
                                delta = Ld[n][p[n]]
                                q[n] += 1
                                rel = delta / (delta + Ld[n][q[n]])
                                o = rawH(n, p) * (1.0 - rel) + rawH(n, q) * rel
                    out[n, i, j, k] = o
    return out


def assert_same_operator(prod_op, ref_op):
    """The product's operator build and the oracle's independent one agree
    bit for bit: every coefficient array, UPML slab, ADE list, excitation
    list and signal, Mur face, RLC list, dT, the probe interval and every
    snapped probe."""
    import oracle
    a = oracle.desc_arrays(prod_op.desc)
    b = oracle.desc_arrays(ref_op.desc)
    assert sorted(a) == sorted(b), (sorted(set(a) ^ set(b)))
    bad = []
    for k in a:
        x, y = a[k], b[k]
        if x.shape != y.shape:
            bad.append((k, "shape", x.shape, y.shape))
            continue
        if x.dtype.kind == "f":
            w = np.uint32 if x.dtype == np.float32 else np.uint64
            neq = x.view(w) != y.view(w)
        else:
            neq = x != y
        if neq.any():
            i = np.nonzero(neq)[0]
            bad.append((k, int(neq.sum()), i[:4].tolist(), x[i[:2]].tolist(), y[i[:2]].tolist()))
    assert not bad, bad
    assert prod_op.dT == ref_op.dT
    assert prod_op.probe_interval == ref_op.probe_interval
    assert prod_op.nyquist == ref_op.nyquist
    # a disabled probe is read by nobody: its type, weight and state are
    # compared, not the placeholder corners each build leaves in it
    def probes(op):
        return [t if t[-1] else (t[0], t[6], t[7]) for t in oracle.probe_tuples(op.probes)]
    assert probes(prod_op) == probes(ref_op)


def oracle_operator(prod_op, threads: int = 0):
    """The oracle's own operator build of the scene `prod_op` was built from,
    checked bitwise against `prod_op`.  Parity tests run the oracle on this
    one, so no parity check rests on the product's operator build."""
    import oracle
    ref = oracle.Operator(prod_op.scene.spec, threads=threads)
    assert_same_operator(prod_op, ref)
    return ref


def oracle_inputs(prod_op):
    """(desc, probes) of the oracle's own operator build of prod_op's scene,
    checked bitwise against prod_op (built once, kept alive with prod_op):
    what the parity tests hand to oracle.run."""
    import os
    ref = getattr(prod_op, "_oracle_op", None)
    if ref is None:
        ref = oracle_operator(prod_op, threads=os.cpu_count() or 1)
        prod_op._oracle_op = ref
    return ref.desc, ref.probes


def with_signal(scene, excite_type: int, f: float = 0.0, function: str = ""):
    """The scene with its Gaussian pulse replaced by another signal of the
    reference: 1 sinusoid of frequency f, 2 Dirac pulse, 3 step (f = f_max),
    10 the custom `function` of t (f = f0)."""
    import copy
    from wipems_gb300 import Scene, SceneSpec
    src = copy.deepcopy(scene.spec)
    sp = SceneSpec(*src["lines"], src["unit"])
    src.update(excite_type=int(excite_type), f0=float(f) if excite_type in (1, 10) else 0.0, fc=0.0,
               f_max=float(f) if excite_type in (2, 3) else 0.0, function=function)
    sp.spec = src
    return Scene.from_spec(sp)
