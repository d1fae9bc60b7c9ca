"""The oracle restatement against the reference's own CPU code (CPU only).

oracle/_ref/libddref.so is the reference's include/Dedispersion.hpp CPU
templates and src/Shifts.cpp compiled unmodified; these tests pin the C
restatement (oracle/dd_oracle.c) and the engine's host-side shift tables to
it bit for bit, on every case the reference defines.
"""
import ctypes as C

import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn

from helpers import elem_count, oracle_run, single_case, step_one_case, step_two_case

F32P = C.POINTER(C.c_float)
U32P = C.POINTER(C.c_uint32)


def ref_shifts(ref, obs, padding, step_two=False):
    out = np.zeros(obs.getNrChannels() + padding + 64, dtype=np.float32)
    fn = ref.ddref_get_shifts_step_two if step_two else ref.ddref_get_shifts
    n = fn(C.byref(obs.c), padding, out.ctypes.data_as(F32P), out.size)
    assert n > 0
    return out[:n]


def ref_single(ref, case):
    out = case.output()
    rc = ref.ddref_dedispersion(C.byref(case.obs.c), case.zapped.ctypes.data_as(U32P),
                                case.zapped.size, case.mapping.ctypes.data_as(U32P),
                                case.mapping.size, C.c_void_p(case.inp.ctypes.data),
                                elem_count(case), out.ctypes.data_as(F32P), out.size,
                                case.shifts.ctypes.data_as(F32P), case.shifts.size, case.padding,
                                case.bits)
    assert rc == 0
    return out


OBSERVATIONS = [
    dict(C=256, fmin=1425.0, bw=0.1953125, tsamp=40.96e-6, S=1024),
    dict(C=1536, fmin=1220.0, bw=0.1953125, tsamp=81.92e-6, S=24576),
    dict(C=384, fmin=1220.0, bw=0.78125, tsamp=81.92e-6, S=8192),
    dict(C=97, fmin=120.0, bw=0.5, tsamp=1e-3, S=333),
]


@pytest.mark.parametrize("o", OBSERVATIONS)
@pytest.mark.parametrize("padding", [0, 64, 128])
def test_shifts_match_reference(engine, oracle, ref, o, padding):
    obs = syn.make_observation(o["C"], o["fmin"], o["bw"], o["tsamp"], o["S"], 8, 0.0, 1.0)
    want = ref_shifts(ref, obs, padding)
    got_lib = dd.getShifts(obs, padding)
    got_oracle = oracle.shifts(obs.c, padding)
    assert want.dtype == got_lib.dtype == np.float32
    np.testing.assert_array_equal(got_lib.view(np.uint32), want.view(np.uint32))
    np.testing.assert_array_equal(got_oracle.view(np.uint32), want.view(np.uint32))
    assert want[o["C"] - 1] == 0.0


@pytest.mark.parametrize("padding", [0, 128])
@pytest.mark.parametrize("sb", [4, 32])
def test_shifts_step_two_match_reference(engine, oracle, ref, padding, sb):
    obs = syn.make_observation(1536, 1220.0, 0.1953125, 81.92e-6, 24576, 32, 0.0, 0.2,
                               subbands=sb, dms1=64, dm_step1=6.4)
    want = ref_shifts(ref, obs, padding, step_two=True)
    np.testing.assert_array_equal(dd.getShiftsStepTwo(obs, padding).view(np.uint32),
                                  want.view(np.uint32))
    np.testing.assert_array_equal(oracle.shifts(obs.c, padding, step_two=True).view(np.uint32),
                                  want.view(np.uint32))
    # subband frequencies: top channel of each subband; the last subband ends at fmax
    assert obs.getSubbandMaxFreq() == obs.getMaxFreq()


CASES_SINGLE = [
    dict(bits=8, padding=0),
    dict(bits=8, padding=64, beams=3, sbeams=5),
    dict(bits=8, padding=128, C=37, D=7, S=61, zap=0.3),
    dict(bits=16, padding=64, beams=2, sbeams=2),
    dict(bits=32, padding=0, beams=2, sbeams=3, dist="gaussian"),
    dict(bits=8, padding=0, dist="constant", mean=10, zap=0.0),
    dict(bits=8, padding=32, first=3.5, step=0.75, D=9),
]


@pytest.mark.parametrize("kw", CASES_SINGLE)
def test_single_step_restatement_matches_reference(engine, oracle, ref, kw):
    case = single_case(seed=3, **kw)
    want = ref_single(ref, case)
    got = oracle_run(oracle, case, threads=2)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("bits", [1, 2, 4])
@pytest.mark.parametrize("padding", [0, 16])
def test_subbyte_restatement_matches_reference(engine, oracle, ref, bits, padding):
    # The reference's sub-byte indexing is only right for beam 0 and rows of
    # S_disp a multiple of 8 / bits (its row length floors); that is the
    # domain checked here.
    case = single_case(C=48, D=10, S=96, bits=bits, padding=padding, beams=1, sbeams=1,
                       seed=5, sdisp_multiple=8 // bits * 8,
                       mapping=np.zeros(dd.pad(48, padding // 4), np.uint32))
    want = ref_single(ref, case)
    got = oracle_run(oracle, case, threads=2)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("padding", [0, 64])
def test_step_one_restatement_matches_reference(engine, oracle, ref, padding):
    case = step_one_case(bits=8, padding=padding, seed=9, beams=2)
    out = case.output()
    z = case.zapped
    rc = ref.ddref_step_one_u8(C.byref(case.obs.c), z.ctypes.data_as(U32P), z.size,
                               C.c_void_p(case.inp.ctypes.data), case.inp.size,
                               out.ctypes.data_as(F32P), out.size,
                               case.shifts.ctypes.data_as(F32P), case.shifts.size, padding)
    assert rc == 0
    got = oracle_run(oracle, case, threads=2)
    np.testing.assert_array_equal(got.view(np.uint32), out.view(np.uint32))


@pytest.mark.parametrize("padding", [0, 64])
@pytest.mark.parametrize("float_values", [False, True])
def test_step_two_restatement_matches_reference(engine, oracle, ref, padding, float_values):
    case = step_two_case(padding=padding, seed=4, beams=2, sbeams=3, float_values=float_values)
    out = case.output()
    m = case.mapping
    rc = ref.ddref_step_two(C.byref(case.obs.c), m.ctypes.data_as(U32P), m.size,
                            case.inp.ctypes.data_as(F32P), case.inp.size,
                            out.ctypes.data_as(F32P), out.size,
                            case.shifts.ctypes.data_as(F32P), case.shifts.size, padding)
    assert rc == 0
    got = oracle_run(oracle, case, threads=2)
    np.testing.assert_array_equal(got.view(np.uint32), out.view(np.uint32))


def test_known_answer_constant_input(engine, oracle):
    # src/DedispersionTest.cpp:210-214: constant 10 gives 10 * (C - zapped) everywhere.
    case = single_case(C=64, D=16, S=128, bits=8, zap=0.25, dist="constant", mean=10)
    got = case.valid(oracle_run(oracle, case))
    live = int((case.zapped[:64] == 0).sum())
    assert np.all(got == 10.0 * live)


@pytest.mark.parametrize("bits", [1, 2, 4])
def test_known_answer_subbyte_constant(engine, oracle, bits):
    # src/DedispersionTest.cpp:222-226: constant bits - 1 gives (bits - 1) * (C - zapped).
    case = single_case(C=40, D=8, S=64, bits=bits, zap=0.2, dist="constant", mean=bits - 1,
                       sdisp_multiple=8)
    got = case.valid(oracle_run(oracle, case))
    live = int((case.zapped[:40] == 0).sum())
    assert np.all(got == float((bits - 1) * live))


def test_known_answer_all_zapped_and_dm_zero(engine, oracle):
    case = single_case(C=32, D=4, S=50, bits=8, zap=1.0)
    assert np.all(case.valid(oracle_run(oracle, case)) == 0.0)
    case = single_case(C=32, D=1, S=50, bits=8, zap=0.0, first=0.0, step=0.0)
    got = case.valid(oracle_run(oracle, case))
    rows = case.inp.reshape(32, -1)[:, :50].astype(np.float64)
    np.testing.assert_array_equal(got[0], rows.sum(axis=0))


def test_known_answer_impulse(engine, oracle):
    # One non-zero sample per channel at t0 + delay(c, dm*): output peaks at dm*.
    case = single_case(C=48, D=20, S=80, bits=8, zap=0.0, dist="constant", mean=0)
    rows = case.inp.reshape(48, -1)
    dm_star, t0 = 13, 17
    a = np.float32(case.obs.getFirstDM()) + np.float32(dm_star) * np.float32(case.obs.getDMStep())
    for c in range(48):
        rows[c, t0 + int(np.float32(a * case.shifts[c]))] = 1
    got = case.valid(oracle_run(oracle, case))
    assert got[dm_star, t0] == 48.0
    assert got.max() == 48.0


def test_fp64_oracle_close_to_float(engine, oracle):
    case = single_case(C=64, D=12, S=100, bits=32, dist="gaussian", mean=5.0, sigma=3.0)
    f32 = case.valid(oracle_run(oracle, case))
    out64 = np.zeros(case.out_elems, dtype=np.float64)
    oracle.dedispersion(case.obs.c, case.zapped, case.mapping, case.inp, out64, case.shifts,
                        case.padding, 32, f64=True)
    f64 = out64.reshape(case.out_rows, case.out_row)[:, :case.nr_samples]
    rel = np.abs(f32 - f64) / np.maximum(np.abs(f64), 1e-30)
    assert rel.max() < 1e-5
