"""Case builders shared by the CPU and GPU tests."""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn


@dataclass
class Case:
    obs: dd.Observation
    mode: int
    bits: int
    padding: int
    shifts: np.ndarray
    zapped: np.ndarray
    mapping: np.ndarray
    inp: np.ndarray
    out_elems: int
    out_row: int
    out_rows: int
    nr_samples: int

    def output(self) -> np.ndarray:
        return np.zeros(self.out_elems, dtype=np.float32)

    def valid(self, out: np.ndarray) -> np.ndarray:
        """[rows, nr_samples] view of the samples the kernels define."""
        return out.reshape(self.out_rows, self.out_row)[:, :self.nr_samples]


def _round_up(v: int, m: int) -> int:
    return -(-v // m) * m


def single_case(C=64, D=24, S=100, bits=8, padding=0, beams=1, sbeams=1, zap=0.1, seed=0,
                first=0.0, step=0.25, fmin=1425.0, bw=0.1953125, tsamp=40.96e-6,
                dist="uniform", mean=128.0, sigma=16.0, sdisp_multiple=1, extra=0,
                mapping=None) -> Case:
    obs = syn.make_observation(C, fmin, bw, tsamp, S, D, first, step, beams=beams,
                               synthesized_beams=sbeams, padding=padding)
    sdisp = _round_up(obs.getNrSamplesPerDispersedBatch() + extra, sdisp_multiple)
    obs.setNrSamplesPerDispersedBatch(sdisp)
    shifts = dd.getShifts(obs, padding)
    z = syn.zapped_mask(C, zap, seed + 7, padding)
    if mapping is None:
        rng = np.random.default_rng(seed + 11)
        row = len(z)
        m = np.zeros((sbeams, row), dtype=np.uint32)
        m[:, :C] = rng.integers(0, beams, size=(sbeams, C))
        mapping = m.reshape(-1)
    inp = syn.make_input(obs, bits, padding, seed, distribution=dist, mean=mean, sigma=sigma)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, bits, padding)
    return Case(obs, dd.DD_SINGLE_STEP, bits, padding, shifts, z, np.asarray(mapping, np.uint32),
                inp, lay.output_bytes // 4, lay.output_row_elems, sbeams * D, S)


def subband_obs(C=96, SB=4, D1=8, step1=2.0, D2=8, step2=0.25, S=100, padding=0, beams=1,
                sbeams=1, fmin=1300.0, bw=0.78125, tsamp=81.92e-6):
    return syn.make_observation(C, fmin, bw, tsamp, S, D2, 0.0, step2, beams=beams,
                                synthesized_beams=sbeams, subbands=SB, dms1=D1, first_dm1=0.0,
                                dm_step1=step1, padding=padding)


def step_one_case(bits=8, padding=0, zap=0.1, seed=0, dist="uniform", sdisp_multiple=1,
                  **kw) -> Case:
    obs = subband_obs(padding=padding, **kw)
    s1d = _round_up(obs.getNrSamplesPerDispersedBatch(True), sdisp_multiple)
    obs.setNrSamplesPerDispersedBatch(s1d, True)
    shifts = dd.getShifts(obs, padding)
    z = syn.zapped_mask(obs.getNrChannels(), zap, seed + 7, padding)
    inp = syn.make_input(obs, bits, padding, seed, mode=dd.DD_STEP_ONE, distribution=dist)
    lay = dd.layout(obs, dd.DD_STEP_ONE, bits, padding)
    rows = obs.getNrBeams() * obs.getNrDMs(True) * obs.getNrSubbands()
    return Case(obs, dd.DD_STEP_ONE, bits, padding, shifts, z, np.zeros(0, np.uint32), inp,
                lay.output_bytes // 4, lay.output_row_elems, rows, obs.getNrSamplesPerBatch(True))


def step_two_case(padding=0, seed=0, float_values=False, **kw) -> Case:
    obs = subband_obs(padding=padding, **kw)
    shifts = dd.getShiftsStepTwo(obs, padding)
    inp = syn.make_input(obs, 32, padding, seed, mode=dd.DD_STEP_TWO)
    if float_values:
        rng = np.random.default_rng(seed + 3)
        inp = (inp + rng.normal(0, 1, size=inp.shape)).astype(np.float32)
    lay = dd.layout(obs, dd.DD_STEP_TWO, 32, padding)
    sb = obs.getNrSynthesizedBeams()
    m = np.zeros((sb, lay.mapping_row_elems), dtype=np.uint32)
    rng = np.random.default_rng(seed + 5)
    m[:, :obs.getNrSubbands()] = rng.integers(0, obs.getNrBeams(), size=(sb, obs.getNrSubbands()))
    rows = sb * obs.getNrDMs(True) * obs.getNrDMs()
    return Case(obs, dd.DD_STEP_TWO, 32, padding, shifts, np.zeros(0, np.uint32), m.reshape(-1),
                inp, lay.output_bytes // 4, lay.output_row_elems, rows, obs.getNrSamplesPerBatch())


def oracle_run(oracle, case: Case, threads=None) -> np.ndarray:
    out = case.output()
    if case.mode == dd.DD_SINGLE_STEP:
        oracle.dedispersion(case.obs.c, case.zapped, case.mapping, case.inp, out, case.shifts,
                            case.padding, case.bits, threads=threads)
    elif case.mode == dd.DD_STEP_ONE:
        oracle.step_one(case.obs.c, case.zapped, case.inp, out, case.shifts, case.padding,
                        case.bits, threads=threads)
    else:
        oracle.step_two(case.obs.c, case.mapping, case.inp, out, case.shifts, case.padding,
                        threads=threads)
    return out


def engine_run(case: Case) -> np.ndarray:
    out = case.output()
    if case.mode == dd.DD_SINGLE_STEP:
        dd.dedispersion(case.obs, case.zapped, case.mapping, case.inp, out, case.shifts,
                        case.padding, case.bits)
    elif case.mode == dd.DD_STEP_ONE:
        dd.subbandDedispersionStepOne(case.obs, case.zapped, case.inp, out, case.shifts,
                                      case.padding, case.bits)
    else:
        dd.subbandDedispersionStepTwo(case.obs, case.mapping, case.inp, out, case.shifts,
                                      case.padding)
    return out


def elem_count(case: Case) -> int:
    """Elements of the input in its storage type."""
    if case.bits == 16:
        return case.inp.nbytes // 2
    if case.bits == 32:
        return case.inp.nbytes // 4
    return case.inp.nbytes
