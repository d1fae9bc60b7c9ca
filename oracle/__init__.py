"""CPU oracle for the dedispersion path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package, and only as the checker (or as the timed CPU baseline); the
engine in ``dedispersion_gb300`` never imports it.

* :data:`restated` -- ``oracle/libddoracle.so``, the C restatement of the
  reference's CPU loops (oracle/dd_oracle.c cites the lines it follows).
* :func:`reference` -- ``oracle/_ref/libddref.so``, the reference's own CPU
  templates compiled unmodified (oracle/Makefile, target ``ref``), present
  only where the reference's sources were available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from .types import DdConf, DdObservation  # noqa: F401  (re-exported for callers)

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "libddoracle.so"
REF_LIB = HERE / "_ref" / "libddref.so"

# Structs are passed by address: either oracle.types' mirrors or the engine's
# own structs of the same layout.
_OBS = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_F32P = C.POINTER(C.c_float)
_F64P = C.POINTER(C.c_double)

_oracle = None
_ref = None


def _f32(a):
    return a.ctypes.data_as(_F32P)


def _u32(a):
    return a.ctypes.data_as(_U32P)


def reference_sources() -> Path | None:
    """Where the reference's sources are: $DD_REFERENCE, else the location
    oracle/Makefile names; None when neither holds include/Dedispersion.hpp
    (always the case on a machine without the reference checkout)."""
    src = os.environ.get("DD_REFERENCE")
    if not src:
        proc = subprocess.run(["make", "-s", "--no-print-directory", "-C", str(HERE),
                               "print-reference"], capture_output=True, text=True)
        src = proc.stdout.strip() if proc.returncode == 0 else ""
    if src and (Path(src) / "include" / "Dedispersion.hpp").exists():
        return Path(src)
    return None


def build(reference: bool = False, verbose: bool = False) -> None:
    """Compile the restatement (oracle/libddoracle.so); with reference=True
    also the reference's own CPU code (oracle/_ref/libddref.so) where its
    sources are present.  Test infrastructure: the engine never calls this."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if reference:
        src = reference_sources()
        if src is not None:
            subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REFERENCE={src}"],
                           check=True)
    if verbose:
        print("built oracle" + (" and oracle/_ref" if REF_LIB.exists() else ""))


def restated() -> C.CDLL:
    """The restatement library (built on first use)."""
    global _oracle
    if _oracle is None:
        if not ORACLE_LIB.exists():
            build()
        h = C.CDLL(str(ORACLE_LIB))
        h.ddo_get_shifts.argtypes = [_OBS, C.c_uint32, _F32P, C.c_size_t]
        h.ddo_get_shifts_step_two.argtypes = [_OBS, C.c_uint32, _F32P, C.c_size_t]
        h.ddo_row_bytes.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        h.ddo_row_bytes.restype = C.c_uint64
        h.ddo_dedispersion.argtypes = [_OBS, _U32P, _U32P, C.c_void_p, _F32P, _F32P, C.c_uint32,
                                       C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]
        h.ddo_dedispersion_f64.argtypes = [_OBS, _U32P, _U32P, C.c_void_p, _F64P, _F32P,
                                           C.c_uint32, C.c_uint32, C.c_int]
        h.ddo_step_one.argtypes = [_OBS, _U32P, C.c_void_p, _F32P, _F32P, C.c_uint32, C.c_uint32,
                                   C.c_int]
        h.ddo_step_two.argtypes = [_OBS, _U32P, _F32P, _F32P, _F32P, C.c_uint32, C.c_int]
        for name in ("ddo_max_freq_c", "ddo_subband_min_freq_c", "ddo_subband_max_freq_c",
                     "ddo_subband_bandwidth_c"):
            getattr(h, name).argtypes = [_OBS]
            getattr(h, name).restype = C.c_float
        _oracle = h
    return _oracle


def reference() -> C.CDLL | None:
    """The reference's own CPU code, or None where it was not built."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            build(reference=True)
        if not REF_LIB.exists():
            return None
        h = C.CDLL(str(REF_LIB))
        h.ddref_get_shifts.argtypes = [_OBS, C.c_uint, _F32P, C.c_size_t]
        h.ddref_get_shifts_step_two.argtypes = [_OBS, C.c_uint, _F32P, C.c_size_t]
        h.ddref_dedispersion.argtypes = [_OBS, _U32P, C.c_size_t, _U32P, C.c_size_t, C.c_void_p,
                                         C.c_size_t, _F32P, C.c_size_t, _F32P, C.c_size_t,
                                         C.c_uint, C.c_uint]
        h.ddref_step_one_u8.argtypes = [_OBS, _U32P, C.c_size_t, C.c_void_p, C.c_size_t, _F32P,
                                        C.c_size_t, _F32P, C.c_size_t, C.c_uint]
        h.ddref_step_two.argtypes = [_OBS, _U32P, C.c_size_t, _F32P, C.c_size_t, _F32P,
                                     C.c_size_t, _F32P, C.c_size_t, C.c_uint]
        h.ddref_read_tuned_conf.argtypes = [C.c_char_p, C.c_char_p, C.c_uint, C.c_void_p,
                                            C.c_char_p, C.c_size_t]
        _ref = h
    return _ref


def row_bytes(samples: int, bits: int, padding: int) -> int:
    return int(restated().ddo_row_bytes(samples, bits, padding))


def shifts(obs: DdObservation, padding: int, step_two: bool = False) -> np.ndarray:
    n = (obs.nr_subbands if step_two else obs.nr_channels) + padding + 8
    out = np.zeros(n, dtype=np.float32)
    fn = restated().ddo_get_shifts_step_two if step_two else restated().ddo_get_shifts
    if fn(C.byref(obs), padding, _f32(out), n) != 0:
        raise ValueError("oracle shift table failed")
    pad = padding // 4
    count = obs.nr_subbands if step_two else obs.nr_channels
    m = count if pad == 0 else -(-count // pad) * pad
    return out[:m].copy()


def dedispersion(obs, zapped, mapping, inp, out, shifts_, padding, bits, dm_begin=0, dm_end=0,
                 threads=None, f64=False):
    """Single step; ``out`` (float32, or float64 with f64=True) filled in place."""
    threads = threads or os.cpu_count() or 1
    z = np.ascontiguousarray(zapped, dtype=np.uint32)
    m = np.ascontiguousarray(mapping, dtype=np.uint32)
    s = np.ascontiguousarray(shifts_, dtype=np.float32)
    inp = np.ascontiguousarray(inp)
    if f64:
        rc = restated().ddo_dedispersion_f64(C.byref(obs), _u32(z), _u32(m),
                                             C.c_void_p(inp.ctypes.data),
                                             out.ctypes.data_as(_F64P), _f32(s), padding, bits,
                                             threads)
    else:
        rc = restated().ddo_dedispersion(C.byref(obs), _u32(z), _u32(m),
                                         C.c_void_p(inp.ctypes.data), _f32(out), _f32(s), padding,
                                         bits, dm_begin, dm_end, threads)
    if rc != 0:
        raise ValueError("oracle dedispersion failed")


def step_one(obs, zapped, inp, out, shifts_, padding, bits, threads=None):
    threads = threads or os.cpu_count() or 1
    z = np.ascontiguousarray(zapped, dtype=np.uint32)
    s = np.ascontiguousarray(shifts_, dtype=np.float32)
    inp = np.ascontiguousarray(inp)
    if restated().ddo_step_one(C.byref(obs), _u32(z), C.c_void_p(inp.ctypes.data), _f32(out),
                               _f32(s), padding, bits, threads) != 0:
        raise ValueError("oracle step one failed")


def step_two(obs, mapping, inp, out, shifts_, padding, threads=None):
    threads = threads or os.cpu_count() or 1
    m = np.ascontiguousarray(mapping, dtype=np.uint32)
    s = np.ascontiguousarray(shifts_, dtype=np.float32)
    inp = np.ascontiguousarray(inp, dtype=np.float32)
    if restated().ddo_step_two(C.byref(obs), _u32(m), _f32(inp), _f32(out), _f32(s), padding,
                               threads) != 0:
        raise ValueError("oracle step two failed")
