"""Generates tests/golden/golden.npz from the reference's own CPU code.

Run here, where the reference's sources are available:

    python tests/golden/make_golden.py

Every case's input is regenerated from its seed by
``dedispersion_gb300.synthetic`` (numpy PCG64, identical on every machine);
the output is computed by ``oracle/_ref/libddref.so`` -- the reference's
include/Dedispersion.hpp CPU templates and src/Shifts.cpp compiled
unmodified -- and stored with a SHA-256 of the input so that a drift of the
generator is caught instead of read as a kernel bug.  The shift tables are
the reference's getShifts / getShiftsStepTwo.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle  # noqa: E402
from helpers import elem_count, single_case, step_one_case, step_two_case  # noqa: E402
from dedispersion_gb300 import synthetic as syn  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"
F32P = C.POINTER(C.c_float)
U32P = C.POINTER(C.c_uint32)

# name -> (builder, kwargs); builders from tests/helpers.py
CASES = {
    "single_u8_multibeam": ("single", dict(C=64, D=24, S=100, bits=8, padding=0, beams=2,
                                           sbeams=3, zap=0.1, seed=101)),
    "single_u8_pad128_ragged": ("single", dict(C=300, D=70, S=700, bits=8, padding=128,
                                               zap=0.05, seed=102, dist="gaussian",
                                               sigma=40.0)),
    "single_u16": ("single", dict(C=40, D=33, S=300, bits=16, padding=64, seed=103)),
    "single_f32": ("single", dict(C=50, D=17, S=211, bits=32, padding=0, seed=104,
                                  dist="gaussian")),
    "single_4bit": ("single", dict(C=48, D=10, S=96, bits=4, padding=16, seed=105,
                                   sdisp_multiple=16, mapping="zeros")),
    "single_2bit": ("single", dict(C=48, D=10, S=96, bits=2, padding=16, seed=106,
                                   sdisp_multiple=32, mapping="zeros")),
    "single_1bit": ("single", dict(C=48, D=10, S=96, bits=1, padding=16, seed=107,
                                   sdisp_multiple=64, mapping="zeros")),
    "step_one_u8": ("one", dict(bits=8, padding=64, seed=108, beams=2)),
    "step_two_f32": ("two", dict(padding=64, seed=109, beams=2, sbeams=3,
                                 float_values=True)),
}


def build_case(kind, kw):
    kw = dict(kw)
    if kw.get("mapping") == "zeros":
        import dedispersion_gb300 as dd
        kw["mapping"] = np.zeros(dd.pad(kw["C"], kw["padding"] // 4), np.uint32)
    if kind == "single":
        return single_case(**kw)
    if kind == "one":
        return step_one_case(**kw)
    return step_two_case(**kw)


def ref_output(ref, case, kind):
    out = case.output()
    if kind == "single":
        rc = ref.ddref_dedispersion(C.byref(case.obs.c), case.zapped.ctypes.data_as(U32P),
                                    case.zapped.size, case.mapping.ctypes.data_as(U32P),
                                    case.mapping.size, C.c_void_p(case.inp.ctypes.data),
                                    elem_count(case), out.ctypes.data_as(F32P), out.size,
                                    case.shifts.ctypes.data_as(F32P), case.shifts.size,
                                    case.padding, case.bits)
    elif kind == "one":
        rc = ref.ddref_step_one_u8(C.byref(case.obs.c), case.zapped.ctypes.data_as(U32P),
                                   case.zapped.size, C.c_void_p(case.inp.ctypes.data),
                                   case.inp.size, out.ctypes.data_as(F32P), out.size,
                                   case.shifts.ctypes.data_as(F32P), case.shifts.size,
                                   case.padding)
    else:
        rc = ref.ddref_step_two(C.byref(case.obs.c), case.mapping.ctypes.data_as(U32P),
                                case.mapping.size, case.inp.ctypes.data_as(F32P), case.inp.size,
                                out.ctypes.data_as(F32P), out.size,
                                case.shifts.ctypes.data_as(F32P), case.shifts.size, case.padding)
    assert rc == 0
    return out


def ref_shifts(ref, obs, padding, step_two=False):
    buf = np.zeros(8192, dtype=np.float32)
    fn = ref.ddref_get_shifts_step_two if step_two else ref.ddref_get_shifts
    n = fn(C.byref(obs.c), padding, buf.ctypes.data_as(F32P), buf.size)
    return buf[:n].copy()


def main():
    ref = oracle.reference()
    if ref is None:
        raise SystemExit("the reference's CPU code is not built (oracle/_ref)")
    arrays, manifest = {}, {}
    for name, (kind, kw) in CASES.items():
        case = build_case(kind, kw)
        arrays[f"{name}__out"] = ref_output(ref, case, kind)
        manifest[name] = {"kind": kind, "kwargs": kw,
                          "input_sha256": hashlib.sha256(case.inp.tobytes()).hexdigest()}
    obs1 = syn.small_observation(128)
    obs2 = syn.large_observation(128)
    obs2s = syn.large_observation(128, subbands=True)
    arrays["shifts_small_pad128"] = ref_shifts(ref, obs1, 128)
    arrays["shifts_large_pad128"] = ref_shifts(ref, obs2, 128)
    arrays["shifts_large_subband_pad128"] = ref_shifts(ref, obs2s, 128)
    arrays["shifts2_large_subband_pad128"] = ref_shifts(ref, obs2s, 128, step_two=True)
    manifest["_dispersed_samples"] = {
        "small": obs1.getNrSamplesPerDispersedBatch(),
        "large": obs2.getNrSamplesPerDispersedBatch(),
        "large_subband_S1": obs2s.getNrSamplesPerBatch(True),
        "large_subband_S1_disp": obs2s.getNrSamplesPerDispersedBatch(True),
    }
    arrays["manifest"] = np.frombuffer(json.dumps(manifest, sort_keys=True).encode(), np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(CASES)} cases)")


if __name__ == "__main__":
    main()
