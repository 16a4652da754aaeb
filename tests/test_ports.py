"""Lumped-port post-processing (ports.py CalcPort / utilities DFT_time2freq
restated): the transform against the reference's own per-frequency loop,
and the wave decomposition on loads with known answers."""
import numpy as np

from wipems_gb300.ports import calc_port, dft_time2freq


def _reference_loop(t, val, freq, signal_type):
    # utilities.py:21-35, element by element
    f_val = np.zeros(len(freq)) * 1j
    for n_f in range(len(freq)):
        f_val[n_f] = np.sum(val * np.exp(-1j * 2 * np.pi * freq[n_f] * t))
    if signal_type == "pulse":
        f_val *= t[1] - t[0]
    else:
        f_val /= len(t)
    return 2 * f_val


def test_dft_matches_reference_loop():
    rng = np.random.default_rng(5)
    t = np.arange(500) * 3.7e-12 + 1.1e-12
    val = rng.standard_normal(500)
    freq = np.linspace(1e9, 20e9, 17)
    for kind in ("pulse", "periodic"):
        np.testing.assert_allclose(dft_time2freq(t, val, freq, kind), _reference_loop(t, val, freq, kind),
                                   rtol=1e-12, atol=1e-12 * np.abs(val).sum())


def test_port_decomposition_known_loads():
    f = np.array([1e9, 2e9])
    i = np.array([0.3 + 0.1j, -0.2 + 0.4j])
    matched = calc_port(f, 50.0 * i, i, 50.0)
    assert np.allclose(matched.s11, 0) and np.allclose(matched.P_ref, 0)
    assert np.allclose(matched.P_acc, matched.P_inc)
    open_ = calc_port(f, np.array([1.0 + 0j, 2j]), np.zeros(2), 50.0)
    assert np.allclose(np.abs(open_.s11), 1) and np.allclose(open_.P_acc, 0)
    short = calc_port(f, np.zeros(2), i, 50.0)
    assert np.allclose(short.s11, -1)
    z = 25.0 + 10j
    load = calc_port(f, z * i, i, 50.0)
    assert np.allclose(load.s11, (z - 50) / (z + 50)) and np.allclose(load.z_in, z)
