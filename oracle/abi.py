"""ORACLE -- test infrastructure only.

ctypes mirrors of the oracle's scene input (operator_oracle.cpp) and of the
engine-description structures of include/wipems_fdtd.h that the oracle's
operator fills (the same memory layout as the product's descriptions, so an
oracle-built description and a product-built one are interchangeable as
inputs of oracle.run)."""
from __future__ import annotations

import ctypes as C

u32 = C.c_uint32
PF = C.POINTER(C.c_float)
PU32 = C.POINTER(C.c_uint32)
PU16 = C.POINTER(C.c_uint16)
D4 = C.c_double * 4
D3 = C.c_double * 3


class OraclePrim(C.Structure):
    _fields_ = [("kind", C.c_int), ("priority", C.c_int), ("start", D3), ("stop", D3),
                ("eps", C.c_double), ("kappa", C.c_double), ("mue", C.c_double), ("sigma", C.c_double),
                ("disp_order", C.c_int), ("eps_plasma_f", D4), ("eps_relax_t", D4), ("eps_pole_f", D4),
                ("mue_plasma_f", D4), ("mue_relax_t", D4), ("mue_pole_f", D4),
                ("ny", C.c_int), ("le_type", C.c_int), ("R", C.c_double), ("C", C.c_double), ("L", C.c_double),
                ("caps", C.c_int), ("exc_type", C.c_int), ("exc_vec", D3), ("delay", C.c_double),
                ("probe_type", C.c_int), ("weight", C.c_double), ("norm_dir", C.c_int)]


class OracleScene(C.Structure):
    _fields_ = [("lines", C.POINTER(C.c_double) * 3), ("num_lines", u32 * 3), ("unit", C.c_double),
                ("bg_eps", C.c_double), ("bg_mue", C.c_double), ("bg_kappa", C.c_double), ("bg_sigma", C.c_double),
                ("bc", C.c_int * 6), ("pml_size", u32 * 6), ("mur_vph", C.c_double * 6),
                ("f0", C.c_double), ("fc", C.c_double), ("nr_ts", u32), ("oversampling", u32),
                ("num_prims", u32), ("prims", C.POINTER(OraclePrim)), ("excite_type", C.c_int),
                ("f_max", C.c_double), ("function", C.c_char_p)]


class OracleOpInfo(C.Structure):
    _fields_ = [("num_lines", u32 * 3), ("dT", C.c_double), ("nyquist", u32), ("probe_interval", u32),
                ("signal_length", u32), ("max_excite_ts", u32), ("num_probes", u32)]


class UpmlDesc(C.Structure):
    _fields_ = [("start", u32 * 3), ("num_lines", u32 * 3),
                ("vv", PF), ("vvfo", PF), ("vvfn", PF), ("ii", PF), ("iifo", PF), ("iifn", PF)]


class AdeDesc(C.Structure):
    _fields_ = [("count", u32), ("pos", PU32 * 3),
                ("volt_on", C.c_int), ("curr_on", C.c_int), ("volt_lor_on", C.c_int), ("curr_lor_on", C.c_int),
                ("v_int", PF), ("v_ext", PF), ("v_lor", PF), ("i_int", PF), ("i_ext", PF), ("i_lor", PF)]


class MurDesc(C.Structure):
    _fields_ = [("ny", C.c_int), ("top", C.c_int), ("line", u32), ("shift", u32), ("n_p", u32), ("n_pp", u32),
                ("coef_p", PF), ("coef_pp", PF), ("start_ts", u32)]


class RlcDesc(C.Structure):
    _fields_ = [("count", u32), ("pos", PU32 * 3), ("dir", C.POINTER(C.c_int)),
                ("ilv", PF), ("i2v", PF), ("vv2", PF), ("vj1", PF), ("vj2", PF), ("vvd", PF),
                ("ib0", PF), ("b1", PF), ("b2", PF)]


class OpDesc(C.Structure):
    _fields_ = [("num_lines", u32 * 3), ("dT", C.c_double),
                ("vv", PF), ("vi", PF), ("ii", PF), ("iv", PF),
                ("num_upml", u32), ("upml", C.POINTER(UpmlDesc)),
                ("num_ade_orders", u32), ("ade", C.POINTER(AdeDesc)),
                ("volt_count", u32), ("volt_index", PU32 * 3), ("volt_dir", PU16), ("volt_amp", PF),
                ("volt_delay", PU32),
                ("curr_count", u32), ("curr_index", PU32 * 3), ("curr_dir", PU16), ("curr_amp", PF),
                ("curr_delay", PU32),
                ("signal_length", u32), ("signal_volt", PF), ("signal_curr", PF), ("signal_period_ts", u32),
                ("lines", C.POINTER(C.c_double) * 3), ("unit", C.c_double),
                ("num_mur", u32), ("mur", C.POINTER(MurDesc)),
                ("rlc", C.POINTER(RlcDesc))]


class ProbeDesc(C.Structure):
    _fields_ = [("type", C.c_int), ("start", u32 * 3), ("stop", u32 * 3),
                ("start_inside", C.c_int * 3), ("stop_inside", C.c_int * 3),
                ("norm_dir", C.c_int), ("weight", C.c_double), ("enabled", C.c_int)]
