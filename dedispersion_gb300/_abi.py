"""ctypes binding of the C ABI declared in include/dedisp_gb300.h.

The shared library is built in-tree (``dedispersion_gb300/libdedisp_gb300.so``,
see ``dedispersion_gb300.build``).  Loading fails loudly when it is missing:
there is no pure-Python or CPU path behind this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libdedisp_gb300.so"

DD_OK = 0
DD_ERR_INVALID_ARGUMENT = -1
DD_ERR_NO_DEVICE = -2
DD_ERR_CUDA = -3
DD_ERR_OUT_OF_MEMORY = -4
DD_ERR_UNSUPPORTED = -5
DD_ERR_TIMEOUT = -6
DD_ERR_FILE = -7
DD_ERR_OVER_BUDGET = -8
DD_ERR_NOT_FOUND = -9

STATUS_NAMES = {
    0: "DD_OK", -1: "DD_ERR_INVALID_ARGUMENT", -2: "DD_ERR_NO_DEVICE", -3: "DD_ERR_CUDA",
    -4: "DD_ERR_OUT_OF_MEMORY", -5: "DD_ERR_UNSUPPORTED", -6: "DD_ERR_TIMEOUT",
    -7: "DD_ERR_FILE", -8: "DD_ERR_OVER_BUDGET", -9: "DD_ERR_NOT_FOUND",
}

DD_SINGLE_STEP = 0
DD_STEP_ONE = 1
DD_STEP_TWO = 2


class DdObservation(C.Structure):
    _fields_ = [
        ("nr_beams", C.c_uint32),
        ("nr_synthesized_beams", C.c_uint32),
        ("nr_channels", C.c_uint32),
        ("nr_subbands", C.c_uint32),
        ("nr_samples_per_batch", C.c_uint32),
        ("nr_samples_per_dispersed_batch", C.c_uint32),
        ("nr_samples_per_batch_subbanding", C.c_uint32),
        ("nr_samples_per_dispersed_batch_subbanding", C.c_uint32),
        ("nr_dms", C.c_uint32),
        ("nr_dms_subbanding", C.c_uint32),
        ("downsampling", C.c_uint32),
        ("nr_zapped_channels", C.c_uint32),
        ("first_dm", C.c_float),
        ("dm_step", C.c_float),
        ("first_dm_subbanding", C.c_float),
        ("dm_step_subbanding", C.c_float),
        ("sampling_time", C.c_float),
        ("min_freq", C.c_float),
        ("channel_bandwidth", C.c_float),
    ]


class DdConf(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in (
        "split_batches", "local_mem", "unroll", "threads_d0", "threads_d1", "threads_d2",
        "items_d0", "items_d1", "items_d2")]


class DdLayout(C.Structure):
    _fields_ = [
        ("input_row_bytes", C.c_uint64),
        ("input_bytes", C.c_uint64),
        ("output_row_elems", C.c_uint64),
        ("output_bytes", C.c_uint64),
        ("mapping_row_elems", C.c_uint64),
        ("zapped_elems", C.c_uint64),
        ("shifts_elems", C.c_uint64),
        ("max_delay", C.c_uint32),
        ("required_dispersed_samples", C.c_uint32),
    ]


_P = C.c_void_p
_OBS = C.POINTER(DdObservation)
_CONF = C.POINTER(DdConf)
_U32P = C.POINTER(C.c_uint32)
_F32P = C.POINTER(C.c_float)

# name -> (restype, argtypes); one line per declaration of include/dedisp_gb300.h
SIGNATURES = {
    "dd_last_error": (C.c_char_p, []),
    "dd_version": (C.c_int, []),
    "dd_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "dd_pad": (C.c_uint64, [C.c_uint64, C.c_uint64]),
    "dd_get_shifts": (C.c_int, [_OBS, C.c_uint32, _F32P, C.c_size_t]),
    "dd_get_shifts_step_two": (C.c_int, [_OBS, C.c_uint32, _F32P, C.c_size_t]),
    "dd_max_freq": (C.c_float, [_OBS]),
    "dd_subband_min_freq": (C.c_float, [_OBS]),
    "dd_subband_max_freq": (C.c_float, [_OBS]),
    "dd_subband_bandwidth": (C.c_float, [_OBS]),
    "dd_get_layout": (C.c_int, [_OBS, C.c_int, C.c_uint32, C.c_uint32, _F32P,
                                C.POINTER(DdLayout)]),
    "dd_default_conf": (C.c_int, [_OBS, C.c_int, C.c_uint32, _CONF]),
    "dd_conf_print": (C.c_int, [_CONF, C.c_char_p, C.c_size_t]),
    "dd_read_tuned_conf": (C.c_int, [C.c_char_p, C.c_char_p, C.c_uint32, _CONF]),
    "dd_write_tuned_conf": (C.c_int, [C.c_char_p, C.c_char_p, C.c_uint32, _CONF]),
    "dd_dedispersion": (C.c_int, [_OBS, _U32P, _U32P, _P, _F32P, _F32P, C.c_uint32,
                                  C.c_uint32]),
    "dd_subband_dedispersion_step_one": (C.c_int, [_OBS, _U32P, _P, _F32P, _F32P,
                                                   C.c_uint32, C.c_uint32]),
    "dd_subband_dedispersion_step_two": (C.c_int, [_OBS, _U32P, _F32P, _F32P, _F32P,
                                                   C.c_uint32]),
    "dd_subband_create": (C.c_int, [C.POINTER(_P), _OBS, C.c_uint32, C.c_uint32, C.c_int]),
    "dd_subband_set_tables": (C.c_int, [_P, _F32P, C.c_size_t, _F32P, C.c_size_t, _U32P,
                                        C.c_size_t, _U32P, C.c_size_t]),
    "dd_subband_run": (C.c_int, [_P, _P, _P, _P]),
    "dd_subband_check": (C.c_int, [_P, _P]),
    "dd_subband_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]),
    "dd_subband_set_pair_kernel": (C.c_int, [_P, C.c_int]),
    "dd_subband_set_overlap": (C.c_int, [_P, C.c_int]),
    "dd_subband_set_chunks": (C.c_int, [_P, C.c_int]),
    "dd_subband_pair_kernel_count": (C.c_int, []),
    "dd_subband_destroy": (C.c_int, [_P]),
    "dd_subband_dedispersion": (C.c_int, [_OBS, _U32P, _U32P, _P, _F32P, _F32P, _F32P,
                                          C.c_uint32, C.c_uint32]),
    "dd_dedispersion_noalloc": (C.c_int, [_OBS, _U32P, _U32P, _P, _F32P, _F32P, C.c_uint32,
                                          C.c_uint32, _P]),
    "dd_plan_create": (C.c_int, [C.POINTER(_P), _OBS, C.c_int, C.c_uint32, C.c_uint32,
                                 _CONF, C.c_int]),
    "dd_kernel_count": (C.c_int, []),
    "dd_kernel_info": (C.c_int, [C.c_int, C.c_char_p, C.c_size_t, _U32P, _CONF]),
    "dd_plan_create_with_kernel": (C.c_int, [C.POINTER(_P), _OBS, C.c_int, C.c_uint32,
                                             C.c_uint32, C.c_int, C.c_int]),
    "dd_plan_set_shifts": (C.c_int, [_P, _F32P, C.c_size_t]),
    "dd_plan_set_zapped": (C.c_int, [_P, _U32P, C.c_size_t]),
    "dd_plan_set_beam_mapping": (C.c_int, [_P, _U32P, C.c_size_t]),
    "dd_plan_run": (C.c_int, [_P, _P, _P, _P]),
    "dd_plan_check": (C.c_int, [_P, _P]),
    "dd_plan_launches": (C.c_int, [_P, _U32P]),
    "dd_plan_get_conf": (C.c_int, [_P, _CONF]),
    "dd_plan_adds": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "dd_plan_set_overlap": (C.c_int, [_P, C.c_int]),
    "dd_plan_set_wait_limit": (C.c_int, [_P, C.c_uint32]),
    "dd_filterbank_info_read": (C.c_int, [C.c_char_p, _P]),
    "dd_filterbank_read": (C.c_int, [C.c_char_p, _P, C.c_uint64, C.c_uint64, _P]),
    "dd_filterbank_observation": (C.c_int, [_P, _P]),
    "dd_dada_info_read": (C.c_int, [C.c_char_p, _P]),
    "dd_dada_read": (C.c_int, [C.c_char_p, _P, C.c_uint64, C.c_uint64, _P]),
    "dd_dada_observation": (C.c_int, [_P, _P]),
    "dd_transpose_time_major": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_int, _P, C.c_uint64,
                                          C.c_uint64, _P]),
    "dd_plan_run_stats": (C.c_int, [_P, _P, _P, _P, _P]),
    "dd_dm_stats_from_accum": (C.c_int, [_P, C.c_size_t, C.c_uint32, _P]),
    "dd_plan_destroy": (C.c_int, [_P]),
    "dd_batch_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "dd_batch_add": (C.c_int, [_P, _OBS, C.c_uint32, C.c_uint32, _F32P, _U32P, _U32P, _P, _P,
                               _U32P]),
    "dd_batch_add_with_kernel": (C.c_int, [_P, _OBS, C.c_uint32, C.c_uint32, _F32P, _U32P,
                                           _U32P, _P, _P, C.c_int, _U32P]),
    "dd_batch_commit": (C.c_int, [_P]),
    "dd_batch_run": (C.c_int, [_P, _P, C.c_int]),
    "dd_batch_check": (C.c_int, [_P, _P]),
    "dd_batch_info": (C.c_int, [_P, _U32P, _U32P, _U32P]),
    "dd_batch_shared": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "dd_batch_set_persistent": (C.c_int, [_P, C.c_int]),
    "dd_batch_destroy": (C.c_int, [_P]),
    "dd_stream_bytes": (C.c_int, [_OBS, C.c_int, C.c_uint32, C.c_uint32, _F32P, _F32P, _U32P,
                                  C.POINTER(C.c_uint64), _U32P]),
    "dd_stream_create": (C.c_int, [C.POINTER(_P), _OBS, C.c_int, C.c_uint32, C.c_uint32, _F32P,
                                   _F32P, _U32P, C.c_int]),
    "dd_stream_buffers": (C.c_int, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "dd_stream_info": (C.c_int, [_P, _U32P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                 _U32P]),
    "dd_stream_push": (C.c_int, [_P, _P]),
    "dd_stream_set_time_major": (C.c_int, [_P, C.c_int]),
    "dd_stream_set_double_buffer": (C.c_int, [_P, C.c_int]),
    "dd_stream_buffer": (C.c_int, [_P, C.c_int, C.POINTER(_P), C.POINTER(_P)]),
    "dd_stream_next_buffer": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "dd_stream_destroy": (C.c_int, [_P]),
    "dd_mlp_create": (C.c_int, [C.POINTER(_P), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64,
                                C.c_int]),
    "dd_mlp_param_count": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "dd_mlp_get_params": (C.c_int, [_P, _F32P, C.c_uint64]),
    "dd_mlp_set_params": (C.c_int, [_P, _F32P, C.c_uint64]),
    "dd_mlp_forward": (C.c_int, [_P, _F32P, C.c_uint32, _F32P]),
    "dd_mlp_gradients": (C.c_int, [_P, _F32P, _F32P, C.c_uint32, _F32P, _F32P]),
    "dd_mlp_train": (C.c_int, [_P, _F32P, _F32P, C.c_uint32, C.c_uint32, C.c_float, _F32P]),
    "dd_mlp_destroy": (C.c_int, [_P]),
    "dd_plan_time": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, _F32P, _F32P]),
    "dd_measure_add_rate": (C.c_int, [C.c_int, C.c_uint32, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]),
}

_lib: C.CDLL | None = None


class DedispersionError(RuntimeError):
    """Raised for every non-zero dd_status; ``status`` holds the code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def lib() -> C.CDLL:
    """The loaded library (loads it on first use; raises if it is not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is not built: run `python -m dedispersion_gb300.build` "
                "(there is no CPU fallback)")
        handle = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status: int) -> None:
    if status != DD_OK:
        msg = lib().dd_last_error().decode(errors="replace")
        raise DedispersionError(status, msg)
