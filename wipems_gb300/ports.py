"""Port post-processing of a lumped port (the reference's python/openEMS
ports.py `Port.CalcPort` / `LumpedPort.CalcPort`, ports.py:103-180, and
utilities.py `DFT_time2freq`, utilities.py:21-35), from either

* the time-domain probe samples the engine recorded (the reference reads
  them back from its probe files and transforms them with DFT_time2freq), or
* the frequency-domain values the engine accumulated on the device
  (Engine.set_frequencies / fd_results), which need no host transform.

`Scene.add_lumped_port` creates the voltage probe "<name>_ut" (weight -1)
and the current probe "<name>_it" (weight = direction) that this reads.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def dft_time2freq(t, val, freq, signal_type: str = "pulse") -> np.ndarray:
    """Single-sided spectrum of a sampled signal at the given frequencies
    (DFT_time2freq): 2 * sum(val * exp(-2 pi i f t)), times the sample step
    for a pulse, divided by the sample count for a periodic signal."""
    t = np.asarray(t, np.float64)
    val = np.asarray(val, np.float64)
    freq = np.atleast_1d(np.asarray(freq, np.float64))
    if len(t) != len(val) or len(freq) == 0:
        raise ValueError("dft_time2freq: t and val must have one length, freq at least one entry")
    f_val = np.exp(-2j * np.pi * np.outer(freq, t)) @ val
    if signal_type == "pulse":
        f_val = f_val * (t[1] - t[0])
    elif signal_type == "periodic":
        f_val = f_val / len(t)
    else:
        raise ValueError(f'unknown signal type "{signal_type}"')
    return 2 * f_val


@dataclass
class PortResult:
    freq: np.ndarray
    uf_tot: np.ndarray
    if_tot: np.ndarray
    uf_inc: np.ndarray
    if_inc: np.ndarray
    uf_ref: np.ndarray
    if_ref: np.ndarray
    P_inc: np.ndarray   # incoming power
    P_ref: np.ndarray   # reflected power
    P_acc: np.ndarray   # accepted power (incoming - reflected)

    @property
    def s11(self) -> np.ndarray:
        return self.uf_ref / self.uf_inc

    @property
    def z_in(self) -> np.ndarray:
        return self.uf_tot / self.if_tot


def calc_port(freq, uf_tot, if_tot, z_ref: float) -> PortResult:
    """Port.CalcPort's wave decomposition for a reference impedance."""
    uf_tot = np.asarray(uf_tot, np.complex128)
    if_tot = np.asarray(if_tot, np.complex128)
    uf_inc = 0.5 * (uf_tot + if_tot * z_ref)
    if_inc = 0.5 * (if_tot + uf_tot / z_ref)
    uf_ref = uf_tot - uf_inc
    if_ref = if_inc - if_tot
    return PortResult(np.asarray(freq, np.float64), uf_tot, if_tot, uf_inc, if_inc, uf_ref, if_ref,
                      0.5 * np.real(uf_inc * np.conj(if_inc)), 0.5 * np.real(uf_ref * np.conj(if_ref)),
                      0.5 * np.real(uf_tot * np.conj(if_tot)))


def _probe_index(names, name):
    try:
        return names.index(name)
    except ValueError:
        raise KeyError(f"no probe named {name!r} (probes: {names})") from None


def lumped_port_td(samples, probe_names, freq, R: float, name: str = "port", ref_impedance=None,
                   signal_type: str = "pulse") -> PortResult:
    """LumpedPort.CalcPort from the engine's time-domain samples: the
    voltage at the sample times, the current at the dual times (t + dT/2),
    each transformed with dft_time2freq; Z_ref defaults to the port's R."""
    iu = _probe_index(list(probe_names), name + "_ut")
    ii = _probe_index(list(probe_names), name + "_it")
    uf = dft_time2freq(samples.times(iu), samples.values[:, iu], freq, signal_type)
    jf = dft_time2freq(samples.times(ii), samples.values[:, ii], freq, signal_type)
    return calc_port(freq, uf, jf, R if ref_impedance is None else ref_impedance)


def lumped_port_fd(fd_values, freq, probe_names, R: float, name: str = "port", ref_impedance=None) -> PortResult:
    """The same decomposition from the device's frequency-domain probe
    values (Engine.fd_results()[0], [probe][frequency])."""
    iu = _probe_index(list(probe_names), name + "_ut")
    ii = _probe_index(list(probe_names), name + "_it")
    return calc_port(freq, fd_values[iu], fd_values[ii], R if ref_impedance is None else ref_impedance)
