"""ctypes mirror of include/wipems_fdtd.h and the loader of libwipems_fdtd.so.

The library is the in-tree build under wipems_gb300/_build.  There is no
fallback: if it is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libwipems_fdtd.so"

u32 = C.c_uint32
PF = C.POINTER(C.c_float)
PU32 = C.POINTER(C.c_uint32)
PU16 = C.POINTER(C.c_uint16)


class FdtdOperatorInfo(C.Structure):
    _fields_ = [("num_lines", u32 * 3), ("dT", C.c_double), ("unit", C.c_double),
                ("nyquist", u32), ("probe_interval", u32), ("signal_length", u32),
                ("max_excite_ts", u32), ("num_upml", u32), ("ade_order", u32),
                ("volt_exc_count", u32), ("curr_exc_count", u32), ("num_probes", u32),
                ("num_cells", C.c_double)]


class FdtdUpmlDesc(C.Structure):
    _fields_ = [("start", u32 * 3), ("num_lines", u32 * 3),
                ("vv", PF), ("vvfo", PF), ("vvfn", PF), ("ii", PF), ("iifo", PF), ("iifn", PF)]


class FdtdAdeDesc(C.Structure):
    _fields_ = [("count", u32), ("pos", PU32 * 3),
                ("volt_on", C.c_int), ("curr_on", C.c_int), ("volt_lor_on", C.c_int), ("curr_lor_on", C.c_int),
                ("v_int", PF), ("v_ext", PF), ("v_lor", PF), ("i_int", PF), ("i_ext", PF), ("i_lor", PF)]


class FdtdMurDesc(C.Structure):
    _fields_ = [("ny", C.c_int), ("top", C.c_int), ("line", u32), ("shift", u32), ("n_p", u32), ("n_pp", u32),
                ("coef_p", PF), ("coef_pp", PF), ("start_ts", u32)]


class FdtdRlcDesc(C.Structure):
    _fields_ = [("count", u32), ("pos", PU32 * 3), ("dir", C.POINTER(C.c_int)),
                ("ilv", PF), ("i2v", PF), ("vv2", PF), ("vj1", PF), ("vj2", PF), ("vvd", PF),
                ("ib0", PF), ("b1", PF), ("b2", PF)]


class FdtdOpDesc(C.Structure):
    _fields_ = [("num_lines", u32 * 3), ("dT", C.c_double),
                ("vv", PF), ("vi", PF), ("ii", PF), ("iv", PF),
                ("num_upml", u32), ("upml", C.POINTER(FdtdUpmlDesc)),
                ("num_ade_orders", u32), ("ade", C.POINTER(FdtdAdeDesc)),
                ("volt_count", u32), ("volt_index", PU32 * 3), ("volt_dir", PU16), ("volt_amp", PF),
                ("volt_delay", PU32),
                ("curr_count", u32), ("curr_index", PU32 * 3), ("curr_dir", PU16), ("curr_amp", PF),
                ("curr_delay", PU32),
                ("signal_length", u32), ("signal_volt", PF), ("signal_curr", PF), ("signal_period_ts", u32),
                ("lines", C.POINTER(C.c_double) * 3), ("unit", C.c_double),
                ("num_mur", u32), ("mur", C.POINTER(FdtdMurDesc)),
                ("rlc", C.POINTER(FdtdRlcDesc))]


class FdtdDumpBox(C.Structure):
    _fields_ = [("field", C.c_int), ("interp", C.c_int), ("start", u32 * 3), ("stop", u32 * 3), ("step", u32 * 3)]


class FdtdSceneDump(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("field", C.c_int), ("interp", C.c_int), ("file_type", C.c_int),
                ("start", C.c_double * 3), ("stop", C.c_double * 3), ("step", u32 * 3)]


class FdtdProbeDesc(C.Structure):
    _fields_ = [("type", C.c_int), ("start", u32 * 3), ("stop", u32 * 3),
                ("start_inside", C.c_int * 3), ("stop_inside", C.c_int * 3),
                ("norm_dir", C.c_int), ("weight", C.c_double), ("enabled", C.c_int)]


class FdtdEngineOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("max_timesteps", u32), ("probe_interval", u32),
                ("use_graphs", C.c_int), ("energy_on_probe", C.c_int), ("tile_y", C.c_int),
                ("x_chunk", C.c_int), ("kernel", C.c_int), ("stages", C.c_int), ("end_crit", C.c_double)]


class FdtdEngineStats(C.Structure):
    _fields_ = [("num_tuples", u32), ("index_bytes", u32), ("num_upml_nodes", u32),
                ("num_ade_nodes", u32), ("padded_nz", u32), ("device_bytes", C.c_uint64),
                ("tile_y", u32), ("x_chunk", u32), ("kernel", u32)]


class FdtdCopInfo(C.Structure):
    _fields_ = [("num_lines", u32 * 3), ("num_tuples_e", u32), ("num_tuples_h", u32), ("index_bytes_e", u32),
                ("index_bytes_h", u32), ("padded_nz", u32), ("num_upml_nodes", u32), ("num_ade_nodes", u32),
                ("geometry_factored", C.c_int), ("trim_e", C.c_int * 3), ("host_bytes", C.c_uint64),
                ("pinned", C.c_int), ("rotation", C.c_int), ("device_lines", u32 * 3)]


class FdtdBatchOpts(C.Structure):
    _fields_ = [("x_chunk", C.c_int), ("stages", C.c_int), ("blocks_per_sm", C.c_int), ("graph_steps", C.c_int),
                ("bin_mib", C.c_int), ("chains", C.c_int), ("tile_y", C.c_int)]


class FdtdXmlInfo(C.Structure):
    _fields_ = [("nr_ts", u32), ("end_crit", C.c_double), ("oversampling", u32), ("excite_type", C.c_int),
                ("f0", C.c_double), ("fc", C.c_double), ("num_properties", u32), ("num_boxes", u32),
                ("num_probes", u32), ("skipped", u32)]


class FdtdServerOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_uint64), ("max_active", u32), ("round_steps", u32),
                ("build_workers", C.c_int), ("build_threads_per_job", C.c_int), ("batch_min_jobs", u32),
                ("batch", FdtdBatchOpts), ("tile_share", u32)]


class FdtdJobOpts(C.Structure):
    _fields_ = [("end_crit", C.c_double), ("max_timesteps", u32), ("probe_interval", u32), ("keep_fields", C.c_int)]


class FdtdJobStatus(C.Structure):
    _fields_ = [("state", C.c_int), ("error", C.c_int), ("timesteps", u32), ("num_samples", u32),
                ("num_probes", u32), ("probe_interval", u32), ("nodes", C.c_uint64), ("num_lines", u32 * 3),
                ("dT", C.c_double), ("footprint", C.c_uint64), ("t_submit", C.c_double), ("t_built", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double)]


class FdtdServerStats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_uint64), ("jobs_admitted", C.c_uint64), ("jobs_done", C.c_uint64),
                ("jobs_failed", C.c_uint64), ("rounds", C.c_uint64), ("rebuilds", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("node_steps", C.c_double), ("gpu_ms", C.c_double),
                ("budget_bytes", C.c_uint64), ("used_bytes", C.c_uint64), ("peak_bytes", C.c_uint64),
                ("active_jobs", u32), ("last_error", C.c_int), ("elapsed_s", C.c_double)]


class FdtdBatchStats(C.Structure):
    _fields_ = [("num_jobs", u32), ("num_groups", u32), ("num_bins", u32), ("total_nodes", C.c_uint64), ("work_items", C.c_uint64),
                ("persistent_blocks", u32), ("device_bytes", C.c_uint64), ("last_ms", C.c_double),
                ("last_launches", C.c_uint64), ("x_chunk", u32)]


class FdtdError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where} failed ({code}): {msg}")
        self.code = code


_lib = None

# (name, restype, argtypes) for every entry point declared in the header.
_P = C.c_void_p
PD = C.POINTER(C.c_double)
SIGNATURES = [
    ("fdtd_last_error", C.c_size_t, [C.c_char_p, C.c_size_t]),
    ("fdtd_scene_create", C.c_int, [PD, u32, PD, u32, PD, u32, C.c_double, C.POINTER(_P)]),
    ("fdtd_scene_destroy", C.c_int, [_P]),
    ("fdtd_scene_set_background", C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_double]),
    ("fdtd_scene_set_boundary", C.c_int, [_P, C.POINTER(C.c_int), PU32]),
    ("fdtd_scene_set_mur_velocity", C.c_int, [_P, C.POINTER(C.c_double)]),
    ("fdtd_scene_set_gauss_excite", C.c_int, [_P, C.c_double, C.c_double, u32]),
    ("fdtd_scene_set_sinus_excite", C.c_int, [_P, C.c_double, u32]),
    ("fdtd_scene_set_dirac_excite", C.c_int, [_P, C.c_double, u32]),
    ("fdtd_scene_set_step_excite", C.c_int, [_P, C.c_double, u32]),
    ("fdtd_scene_set_custom_excite", C.c_int, [_P, C.c_char_p, C.c_double, C.c_double, u32]),
    ("fdtd_scene_set_oversampling", C.c_int, [_P, u32]),
    ("fdtd_scene_add_material", C.c_int, [_P, C.c_int, PD, PD, C.c_double, C.c_double, C.c_double, C.c_double]),
    ("fdtd_scene_add_metal", C.c_int, [_P, C.c_int, PD, PD]),
    ("fdtd_scene_add_lumped", C.c_int, [_P, C.c_int, PD, PD, C.c_int, C.c_double, C.c_double, C.c_int]),
    ("fdtd_scene_add_lumped_rlc", C.c_int, [_P, C.c_int, PD, PD, C.c_int, C.c_int, C.c_double, C.c_double,
                                            C.c_double, C.c_int]),
    ("fdtd_scene_add_excitation", C.c_int, [_P, C.c_int, PD, PD, C.c_int, PD, C.c_double]),
    ("fdtd_scene_add_lorentz", C.c_int, [_P, C.c_int, PD, PD, C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_int, PD, PD, PD]),
    ("fdtd_scene_add_lorentz_material", C.c_int, [_P, C.c_int, PD, PD, C.c_double, C.c_double, C.c_double,
                                                  C.c_double, C.c_int, PD, PD, PD, PD, PD, PD]),
    ("fdtd_scene_add_probe", C.c_int, [_P, C.c_int, PD, PD, C.c_double, C.c_int]),
    ("fdtd_operator_build", C.c_int, [_P, C.c_int, C.POINTER(_P)]),
    ("fdtd_operator_destroy", C.c_int, [_P]),
    ("fdtd_operator_get_info", C.c_int, [_P, C.POINTER(FdtdOperatorInfo)]),
    ("fdtd_operator_describe", C.c_int, [_P, C.POINTER(FdtdOpDesc)]),
    ("fdtd_operator_get_probe", C.c_int, [_P, u32, C.POINTER(FdtdProbeDesc)]),
    ("fdtd_compress", C.c_int, [C.POINTER(FdtdOpDesc), C.POINTER(_P)]),
    ("fdtd_compress_ex", C.c_int, [C.POINTER(FdtdOpDesc), C.c_int, C.POINTER(_P)]),
    ("fdtd_compress_rot", C.c_int, [C.POINTER(FdtdOpDesc), C.c_int, C.c_int, C.POINTER(_P)]),
    ("fdtd_cop_destroy", C.c_int, [_P]),
    ("fdtd_cop_get_info", C.c_int, [_P, C.POINTER(FdtdCopInfo)]),
    ("fdtd_cop_expand", C.c_int, [_P, PF, PF, PF, PF, PU32, PU32]),
    ("fdtd_cop_expand_ext", C.c_int, [_P, C.c_int, PF, PF]),
    ("fdtd_cop_expand_ade", C.c_int, [_P, C.c_int, C.c_int, PF]),
    ("fdtd_engine_create", C.c_int, [C.POINTER(FdtdOpDesc), C.POINTER(FdtdEngineOpts), C.POINTER(_P)]),
    ("fdtd_engine_create_compressed", C.c_int, [_P, C.POINTER(FdtdEngineOpts), C.POINTER(_P)]),
    ("fdtd_engine_reset", C.c_int, [_P]),
    ("fdtd_engine_destroy", C.c_int, [_P]),
    ("fdtd_engine_add_probe", C.c_int, [_P, C.POINTER(FdtdProbeDesc), PU32]),
    ("fdtd_engine_iterate", C.c_int, [_P, u32]),
    ("fdtd_engine_iterate_async", C.c_int, [_P, u32]),
    ("fdtd_engine_wait", C.c_int, [_P]),
    ("fdtd_engine_query", C.c_int, [_P, C.POINTER(C.c_int)]),
    ("fdtd_engine_set_fd", C.c_int, [_P, PD, u32, u32]),
    ("fdtd_engine_checkpoint", C.c_int, [_P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    ("fdtd_engine_restore", C.c_int, [_P, _P, C.c_uint64]),
    ("fdtd_engine_read_fd", C.c_int, [_P, PD, PU32]),
    ("fdtd_engine_done", C.c_int, [_P, C.POINTER(C.c_int)]),
    ("fdtd_engine_num_timesteps", C.c_int, [_P, PU32]),
    ("fdtd_engine_num_samples", C.c_int, [_P, PU32]),
    ("fdtd_engine_read_samples", C.c_int, [_P, u32, u32, PU32, PD, PD]),
    ("fdtd_engine_energy", C.c_int, [_P, PD]),
    ("fdtd_engine_get_fields", C.c_int, [_P, PF, PF]),
    ("fdtd_engine_get_volt", C.c_int, [_P, u32, u32, u32, u32, PF]),
    ("fdtd_engine_get_curr", C.c_int, [_P, u32, u32, u32, u32, PF]),
    ("fdtd_engine_set_volt", C.c_int, [_P, u32, u32, u32, u32, C.c_float]),
    ("fdtd_engine_set_curr", C.c_int, [_P, u32, u32, u32, u32, C.c_float]),
    ("fdtd_engine_probe_now", C.c_int, [_P, C.POINTER(FdtdProbeDesc), C.POINTER(C.c_double)]),
    ("fdtd_engine_get_stats", C.c_int, [_P, C.POINTER(FdtdEngineStats)]),
    ("fdtd_engine_last_timing", C.c_int, [_P, PD, C.POINTER(C.c_uint64)]),
    ("fdtd_engine_profile_kernels", C.c_int, [_P, u32, PD, PD]),
    ("fdtd_field_energy_static", C.c_int, [_P, _P, PU32, u32, _P, _P]),
    ("fdtd_scene_load_xml", C.c_int, [C.c_char_p, C.POINTER(_P), C.POINTER(FdtdXmlInfo)]),
    ("fdtd_scene_load_xml_file", C.c_int, [C.c_char_p, C.POINTER(_P), C.POINTER(FdtdXmlInfo)]),
    ("fdtd_batch_create", C.c_int, [C.POINTER(_P), u32, C.POINTER(FdtdBatchOpts), C.POINTER(_P)]),
    ("fdtd_batch_accepts", C.c_int, [_P, C.POINTER(C.c_int)]),
    ("fdtd_engine_dump_field", C.c_int, [_P, C.POINTER(FdtdDumpBox), PF, C.c_uint64, PU32]),
    ("fdtd_scene_num_dumps", C.c_int, [_P, PU32]),
    ("fdtd_scene_get_dump", C.c_int, [_P, u32, C.POINTER(FdtdSceneDump)]),
    ("fdtd_batch_iterate", C.c_int, [_P, u32]),
    ("fdtd_batch_info", C.c_int, [_P, C.POINTER(FdtdBatchStats)]),
    ("fdtd_batch_destroy", C.c_int, [_P]),
    ("fdtd_server_create", C.c_int, [C.POINTER(FdtdServerOpts), C.POINTER(_P)]),
    ("fdtd_server_submit", C.c_int, [_P, _P, C.POINTER(FdtdJobOpts), C.POINTER(C.c_uint64)]),
    ("fdtd_server_job_status", C.c_int, [_P, C.c_uint64, C.POINTER(FdtdJobStatus)]),
    ("fdtd_server_wait", C.c_int, [_P, C.c_uint64, C.c_double]),
    ("fdtd_server_read_samples", C.c_int, [_P, C.c_uint64, PU32, PD, PD]),
    ("fdtd_server_probe_types", C.c_int, [_P, C.c_uint64, C.POINTER(C.c_int), u32]),
    ("fdtd_server_get_fields", C.c_int, [_P, C.c_uint64, PF, PF]),
    ("fdtd_server_release", C.c_int, [_P, C.c_uint64]),
    ("fdtd_server_get_stats", C.c_int, [_P, C.POINTER(FdtdServerStats)]),
    ("fdtd_server_destroy", C.c_int, [_P]),
]


def lib() -> C.CDLL:
    """Loads libwipems_fdtd.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists() or os.environ.get("WIPEMS_REBUILD"):
        from . import build as _build
        _build.build()
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: the CUDA engine library was not built")
    L = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(4096)
    lib().fdtd_last_error(buf, 4096)
    return buf.value.decode(errors="replace")


def check(rc: int, where: str) -> None:
    if rc != 0:
        raise FdtdError(rc, where, last_error())
