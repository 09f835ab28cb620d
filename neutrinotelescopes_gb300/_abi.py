"""ctypes view of the C ABI in include/ntp.h and the loader of libntp.so.

The library is the only compute path: if it is missing or fails to load,
every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libntp.so"

NTP_ABI_VERSION = 2

# ntp_status
NTP_OK = 0
NTP_ERR_INVALID = 1
NTP_ERR_OVERFLOW = 2
NTP_ERR_CUDA = 3
NTP_ERR_NOT_READY = 4
NTP_ERR_TIMEOUT = 5
NTP_ERR_NOMEM = 6

# ntp_source_kind
SRC_POINT_ISOTROPIC = 0
SRC_POINT_TIME_RANGE = 1
SRC_AXICONE = 2
SRC_PENCIL = 3
SRC_EXTENDED_CHERENKOV = 4
SRC_POINT_CHERENKOV = 5
SRC_CHERENKOV_TRACK = 6

# ntp_target_kind
TARGET_SPHERE = 0
TARGET_MULTI_PMT = 1

# ntp_spectrum_kind
SPEC_MONOCHROMATIC = 0
SPEC_TABLE_LINEAR = 1
SPEC_TABLE_TEXTURE = 2
SPEC_INV_SQUARE = 3

# ntp_flow_input
FLOW_INPUT_FEATURES = 0
FLOW_INPUT_DERIVED = 1

# ntp_hit_policy / flags
HIT_FIRST_IN_LIST = 0
HIT_NEAREST = 1
FLAG_EXACT_POLE_ROTATION = 1
FLAG_PLAIN_SCAN = 2


class NtpSource(C.Structure):
    _fields_ = [
        ("position", C.c_float * 3),
        ("time", C.c_float),
        ("direction", C.c_float * 3),
        ("angle", C.c_float),
        ("photons", C.c_uint64),
        ("kind", C.c_int32),
        ("time_end", C.c_float),
        ("long_a", C.c_float),
        ("long_b", C.c_float),
        ("long_lrad", C.c_float),
        ("length", C.c_float),
    ]


class NtpTarget(C.Structure):
    _fields_ = [
        ("position", C.c_float * 3),
        ("radius", C.c_float),
        ("module_id", C.c_uint32),
        ("kind", C.c_int32),
        ("pmt_area", C.c_float),
        ("n_pmts", C.c_int32),
        ("pmt_offset", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class NtpMediumDesc(C.Structure):
    _fields_ = [
        ("n_knots", C.c_int32),
        ("wl_min", C.c_float),
        ("wl_max", C.c_float),
        ("ref_index", C.POINTER(C.c_float)),
        ("group_velocity", C.POINTER(C.c_float)),
        ("scattering_length", C.POINTER(C.c_float)),
        ("n_abs_knots", C.c_int32),
        ("abs_wavelength", C.POINTER(C.c_float)),
        ("abs_length", C.POINTER(C.c_float)),
        ("hg_g", C.c_float),
        ("rayleigh_fraction", C.c_float),
    ]


class NtpSpectrumDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("n_knots", C.c_int32),
        ("icdf_knots", C.POINTER(C.c_float)),
        ("wl_min", C.c_float),
        ("wl_max", C.c_float),
        ("wavelength", C.c_float),
    ]


class NtpPropOpts(C.Structure):
    _fields_ = [
        ("max_steps", C.c_int32),
        ("hit_policy", C.c_int32),
        ("flags", C.c_int32),
        ("reserved", C.c_int32),
        ("stream", C.c_void_p),
    ]


class NtpRunStats(C.Structure):
    _fields_ = [
        ("photons", C.c_uint64),
        ("hits", C.c_uint64),
        ("photon_steps", C.c_uint64),
        ("grid", C.c_int32),
        ("block", C.c_int32),
        ("chunk", C.c_uint64),
    ]


class NtpServerConfig(C.Structure):
    _fields_ = [
        ("hbm_budget_bytes", C.c_uint64),
        ("seed", C.c_uint64),
        ("max_events_per_batch", C.c_int32),
        ("max_steps", C.c_int32),
        ("hit_policy", C.c_int32),
        ("flags", C.c_int32),
        ("reserve_hits_per_photon", C.c_double),
        ("min_reserve_hits", C.c_uint64),
        ("max_batch_photons", C.c_uint64),
        ("chunk_photons", C.c_uint64),
    ]


class NtpEventResult(C.Structure):
    _fields_ = [
        ("event_id", C.c_uint32),
        ("status", C.c_int32),
        ("n_hits", C.c_uint64),
        ("n_photons", C.c_uint64),
        ("hits", C.c_void_p),
        ("t_submit", C.c_double),
        ("t_launch", C.c_double),
        ("t_done", C.c_double),
        ("reruns", C.c_int32),
        ("batch_events", C.c_int32),
    ]


class NtpServerStats(C.Structure):
    _fields_ = [
        ("queued", C.c_uint64),
        ("running", C.c_uint64),
        ("completed", C.c_uint64),
        ("released", C.c_uint64),
        ("batches", C.c_uint64),
        ("photons", C.c_uint64),
        ("arena_hits", C.c_uint64),
        ("arena_reserved_hits", C.c_uint64),
        ("clock", C.c_double),
    ]


class NtpSummarySpec(C.Structure):
    _fields_ = [
        ("max_pmts", C.c_int32),
        ("n_bins", C.c_int32),
        ("t_min", C.c_float),
        ("t_max", C.c_float),
        ("use_time_residual", C.c_int32),
        ("source_position", C.c_float * 3),
        ("n800", C.c_float),
    ]


class NtpFlowConfig(C.Structure):
    _fields_ = [
        ("batch_capacity", C.c_int32),
        ("n_layers", C.c_int32),
        ("n_bins", C.c_int32),
        ("t_min", C.c_float),
        ("t_max", C.c_float),
        ("lr", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("eps", C.c_float),
        ("grad_clip", C.c_float),
        ("count_weight", C.c_float),
        ("seed", C.c_uint64),
        ("input_columns", C.c_int32),
        ("reserved", C.c_int32),
    ]


class NtpTableSpec(C.Structure):
    _fields_ = [
        ("n_sims", C.c_int32),
        ("n_orientations", C.c_int32),
        ("max_rows_per_group", C.c_int32),
        ("zero_rows", C.c_int32),
        ("downsample", C.c_double),
        ("n800", C.c_float),
        ("reserved", C.c_int32),
        ("seed", C.c_uint64),
    ]


assert C.sizeof(NtpSource) == 64
assert C.sizeof(NtpTarget) == 48

# ntp_hit as a numpy record (64 bytes)
HIT_DTYPE = np.dtype(
    [
        ("position", np.float32, (3,)),
        ("time", np.float32),
        ("direction", np.float32, (3,)),
        ("wavelength", np.float32),
        ("initial_direction", np.float32, (3,)),
        ("dist_travelled", np.float32),
        ("module_id", np.uint32),
        ("source_index", np.uint32),
        ("photon_index", np.uint64),
    ],
    align=True,
)
assert HIT_DTYPE.itemsize == 64

# every symbol include/ntp.h declares
EXPORTED = (
    "ntp_abi_version",
    "ntp_create",
    "ntp_destroy",
    "ntp_last_error",
    "ntp_set_medium",
    "ntp_set_spectrum",
    "ntp_set_targets",
    "ntp_propagate",
    "ntp_propagate_noalloc",
    "ntp_get_run_stats",
    "ntp_make_hits",
    "ntp_calc_total_weight",
    "ntp_set_wavelength_acceptance",
    "ntp_calc_time_residual",
    "ntp_pmt_summary",
    "ntp_resample",
    "ntp_make_table",
    "ntp_event_conditions",
    "ntp_gemm_bf16",
    "ntp_gemm_set_wait_limit",
    "ntp_flow_create",
    "ntp_flow_destroy",
    "ntp_flow_last_error",
    "ntp_flow_get_layout",
    "ntp_flow_set_params",
    "ntp_flow_get_params",
    "ntp_flow_set_lr",
    "ntp_flow_train_step",
    "ntp_flow_train_steps",
    "ntp_flow_mixture_cdf",
    "ntp_flow_sample_resume",
    "ntp_flow_forward",
    "ntp_flow_head",
    "ntp_flow_evaluate",
    "ntp_flow_sample",
    "ntp_flow_sample_expec",
    "ntp_flow_log_expectation",
    "ntp_flow_evaluate_grid",
    "ntp_server_create",
    "ntp_server_destroy",
    "ntp_server_submit",
    "ntp_server_poll",
    "ntp_server_copy_hits",
    "ntp_server_release",
    "ntp_server_get_stats",
)

_lib = None
_lock = threading.Lock()


def _declare(lib: C.CDLL) -> None:
    vp, i32, u64 = C.c_void_p, C.c_int32, C.c_uint64
    lib.ntp_abi_version.restype = C.c_int
    lib.ntp_create.argtypes = [C.c_int, C.POINTER(vp)]
    lib.ntp_create.restype = C.c_int
    lib.ntp_destroy.argtypes = [vp]
    lib.ntp_destroy.restype = None
    lib.ntp_last_error.argtypes = [vp]
    lib.ntp_last_error.restype = C.c_char_p
    lib.ntp_set_medium.argtypes = [vp, C.POINTER(NtpMediumDesc)]
    lib.ntp_set_spectrum.argtypes = [vp, C.POINTER(NtpSpectrumDesc)]
    lib.ntp_set_targets.argtypes = [vp, C.POINTER(NtpTarget), i32, C.POINTER(C.c_float), i32]
    lib.ntp_propagate.argtypes = [vp, C.POINTER(NtpSource), i32, u64, C.POINTER(NtpPropOpts), vp, u64, i32,
                                  C.POINTER(u64), C.POINTER(u64)]
    lib.ntp_propagate_noalloc.argtypes = [C.POINTER(NtpMediumDesc), C.POINTER(NtpSpectrumDesc), C.POINTER(NtpTarget),
                                          i32, C.POINTER(NtpSource), i32, u64, C.POINTER(NtpPropOpts), vp, u64,
                                          C.POINTER(u64), C.POINTER(u64)]
    lib.ntp_get_run_stats.argtypes = [vp, C.POINTER(NtpRunStats)]
    lib.ntp_make_hits.argtypes = [vp, vp, u64, C.POINTER(C.c_double), vp, i32, vp]
    lib.ntp_calc_total_weight.argtypes = [vp, vp, u64, vp, vp, vp, vp, i32, vp]
    lib.ntp_set_wavelength_acceptance.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), i32]
    lib.ntp_calc_time_residual.argtypes = [vp, vp, u64, C.POINTER(C.c_float), C.c_float, vp, i32, vp]
    lib.ntp_pmt_summary.argtypes = [vp, vp, u64, C.POINTER(C.c_double), C.POINTER(NtpSummarySpec), vp, vp, vp, i32,
                                    vp]
    lib.ntp_pmt_summary.restype = C.c_int
    lib.ntp_resample.argtypes = [vp, vp, u64, vp, vp, vp, i32, C.c_double, u64, vp, vp, vp, u64, C.POINTER(u64),
                                 i32, vp]
    lib.ntp_resample.restype = C.c_int
    lib.ntp_gemm_bf16.argtypes = [vp, i32, vp, i32, vp, i32, i32, i32, i32, vp, i32, i32, i32, vp]
    lib.ntp_gemm_bf16.restype = C.c_int
    lib.ntp_gemm_set_wait_limit.argtypes = [u64, i32]
    lib.ntp_gemm_set_wait_limit.restype = C.c_int
    lib.ntp_make_table.argtypes = [vp, vp, u64, vp, C.POINTER(NtpSource), C.POINTER(C.c_float),
                                   C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(NtpTableSpec), vp, vp, vp,
                                   vp, vp, u64, C.POINTER(u64), vp, vp, vp, vp, vp]
    lib.ntp_make_table.restype = C.c_int
    lib.ntp_event_conditions.argtypes = [vp, C.POINTER(NtpSource), C.POINTER(C.c_float), vp, i32, C.c_float,
                                         C.c_float, C.c_float, vp, vp, vp, vp, vp, vp, u64, C.POINTER(u64), vp, vp,
                                         vp]
    lib.ntp_event_conditions.restype = C.c_int
    lib.ntp_flow_create.argtypes = [i32, C.POINTER(NtpFlowConfig), C.POINTER(vp)]
    lib.ntp_flow_destroy.argtypes = [vp]
    lib.ntp_flow_destroy.restype = None
    lib.ntp_flow_last_error.argtypes = [vp]
    lib.ntp_flow_last_error.restype = C.c_char_p
    lib.ntp_flow_get_layout.argtypes = [vp, C.POINTER(u64), C.POINTER(i32), C.POINTER(i32)]
    lib.ntp_flow_set_params.argtypes = [vp, vp, u64]
    lib.ntp_flow_get_params.argtypes = [vp, vp, u64, i32]
    lib.ntp_flow_set_lr.argtypes = [vp, C.c_float]
    lib.ntp_flow_set_lr.restype = C.c_int
    lib.ntp_flow_train_step.argtypes = [vp, vp, vp, vp, vp, i32, i32, i32, C.POINTER(C.c_double)]
    lib.ntp_flow_train_steps.argtypes = [vp, vp, vp, vp, vp, vp, i32, i32, i32, i32, vp]
    lib.ntp_flow_mixture_cdf.argtypes = [vp, vp, i32, vp, vp, vp, u64, vp, i32]
    lib.ntp_flow_forward.argtypes = [vp, vp, i32, vp]
    lib.ntp_flow_head.argtypes = [vp, vp, vp, vp, vp, vp, i32, C.POINTER(C.c_double), vp]
    lib.ntp_flow_evaluate.argtypes = [vp, vp, i32, vp, vp, u64, vp, vp, i32]
    lib.ntp_flow_sample.argtypes = [vp, vp, i32, vp, u64, vp, vp, vp, u64, C.POINTER(u64), i32]
    lib.ntp_flow_sample_expec.argtypes = [vp, vp, i32, vp, u64, vp, vp, vp, vp, u64, C.POINTER(u64), i32]
    lib.ntp_flow_sample_resume.argtypes = [vp, vp, vp, u64, C.POINTER(u64), i32]
    lib.ntp_flow_log_expectation.argtypes = [vp, vp, i32, vp, i32]
    lib.ntp_flow_evaluate_grid.argtypes = [vp, vp, i32, vp, i32, vp, vp, i32]
    for name in ("ntp_flow_create", "ntp_flow_get_layout", "ntp_flow_set_params", "ntp_flow_get_params",
                 "ntp_flow_train_step", "ntp_flow_forward", "ntp_flow_head", "ntp_flow_evaluate",
                 "ntp_flow_sample", "ntp_flow_evaluate_grid", "ntp_flow_train_steps", "ntp_flow_mixture_cdf",
                 "ntp_flow_sample_resume", "ntp_flow_sample_expec", "ntp_flow_log_expectation"):
        getattr(lib, name).restype = C.c_int
    lib.ntp_server_create.argtypes = [vp, C.POINTER(NtpServerConfig), C.POINTER(vp)]
    lib.ntp_server_destroy.argtypes = [vp]
    lib.ntp_server_destroy.restype = None
    lib.ntp_server_submit.argtypes = [vp, C.c_uint32, C.POINTER(NtpSource)]
    lib.ntp_server_poll.argtypes = [vp, C.POINTER(NtpEventResult), i32, i32]
    lib.ntp_server_poll.restype = i32
    lib.ntp_server_copy_hits.argtypes = [vp, C.c_uint32, vp, u64, C.POINTER(u64)]
    lib.ntp_server_release.argtypes = [vp, C.c_uint32]
    lib.ntp_server_get_stats.argtypes = [vp, C.POINTER(NtpServerStats)]
    for name in ("ntp_server_create", "ntp_server_submit", "ntp_server_copy_hits", "ntp_server_release",
                 "ntp_server_get_stats"):
        getattr(lib, name).restype = C.c_int
    for name in ("ntp_set_medium", "ntp_set_spectrum", "ntp_set_targets", "ntp_propagate", "ntp_propagate_noalloc",
                 "ntp_get_run_stats",
                 "ntp_make_hits",
                 "ntp_calc_total_weight", "ntp_set_wavelength_acceptance", "ntp_calc_time_residual"):
        getattr(lib, name).restype = C.c_int


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Loads libntp.so (building nothing); raises if it is absent.  The
    NTP_LIBRARY environment variable, when set, names the library to load
    instead of the in-tree build."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else Path(os.environ.get("NTP_LIBRARY") or LIB_PATH)
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()' or python neutrinotelescopes_gb300/build.py)"
            )
        lib = C.CDLL(str(p))
        _declare(lib)
        if lib.ntp_abi_version() != NTP_ABI_VERSION:
            raise RuntimeError(f"libntp.so ABI {lib.ntp_abi_version()} != {NTP_ABI_VERSION}")
        if path is None:
            _lib = lib
        return lib


class NtpError(RuntimeError):
    """A libntp call returned a status other than NTP_OK."""

    def __init__(self, status: int, message: str):
        super().__init__(f"libntp status {status}: {message}")
        self.status = status


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))
