"""The 1536-channel x 2048-DM x 24576-sample workload at full size on the GPU.

The CPU oracle (include/Dedispersion.hpp:70-109, threaded over DMs) checks
every one of the 2048 DM rows sample by sample; size-independent properties
check the same output again: the sum of each DM row equals a per-channel
prefix-sum identity computed exactly in integers (a checksum of checksums),
and every injected dispersed pulse peaks at its DM.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

PADDING = 128


@pytest.fixture(scope="module")
def large(gpu):
    obs = syn.large_observation(PADDING)
    shifts = dd.getShifts(obs, PADDING)
    zapped = syn.zapped_mask(1536, 0.05, 7, PADDING)
    mapping = syn.identity_mapping(obs, PADDING)
    inp = syn.make_input(obs, 8, PADDING, seed=1, mean=128.0, sigma=20.0, pulses=20, shifts=shifts)
    out = syn.output_buffer(obs, dd.DD_SINGLE_STEP, PADDING)
    dd.dedispersion(obs, zapped, mapping, inp, out, shifts, PADDING, 8)
    return obs, shifts, zapped, mapping, inp, out


def delays(obs, shifts):
    D = obs.getNrDMs()
    dm = (np.float32(obs.getFirstDM()) +
          np.arange(D, dtype=np.float32) * np.float32(obs.getDMStep())).astype(np.float32)
    return (dm[:, None] * shifts[None, :obs.getNrChannels()].astype(np.float32)).astype(np.uint32)


def test_every_dm_row_matches_oracle(large, oracle):
    obs, shifts, zapped, mapping, inp, out = large
    S, row = obs.getNrSamplesPerBatch(), dd.pad(obs.getNrSamplesPerBatch(), PADDING // 4)
    ref = np.zeros_like(out)
    oracle.dedispersion(obs.c, zapped, mapping, inp, ref, shifts, PADDING, 8, 0, obs.getNrDMs())
    got = out.reshape(-1, row)[:, :S]
    want = ref.reshape(-1, row)[:, :S]
    bad = np.flatnonzero((got.view(np.uint32) != want.view(np.uint32)).any(axis=1))
    assert bad.size == 0, f"DM rows differing from the oracle: {bad[:16]}"


def test_every_dm_row_sum(large):
    """sum_t out[d][t] = sum_c (P_c[S + delay(c, d)] - P_c[delay(c, d)]), P_c the
    prefix sum of channel c: exact integers for all 2048 rows."""
    obs, shifts, zapped, mapping, inp, out = large
    C, S = obs.getNrChannels(), obs.getNrSamplesPerBatch()
    rowb = dd.pad(obs.getNrSamplesPerDispersedBatch(), PADDING)
    rows = inp.reshape(C, rowb).astype(np.int64)
    prefix = np.zeros((C, rowb + 1), np.int64)
    np.cumsum(rows, axis=1, out=prefix[:, 1:])
    dl = delays(obs, shifts).astype(np.int64)  # [D][C]
    live = zapped[:C] == 0
    ch = np.arange(C)[None, :]
    want = ((prefix[ch, S + dl] - prefix[ch, dl]) * live[None, :]).sum(axis=1)
    row = dd.pad(S, PADDING // 4)
    got = out.reshape(-1, row)[:, :S].astype(np.float64).sum(axis=1)
    assert np.array_equal(got.astype(np.int64), want)


def test_injected_pulses_peak_at_their_dm(large):
    obs, shifts, zapped, mapping, inp, out = large
    S = obs.getNrSamplesPerBatch()
    row = dd.pad(S, PADDING // 4)
    grid = out.reshape(-1, row)[:, :S]
    # the strongest pixel of the DM-time plane is one of the injected pulses:
    # the pulses are regenerated with the generator's seed
    rng_vals = np.zeros((1, 1536, obs.getNrSamplesPerDispersedBatch()), np.uint8)
    pulses = syn.inject_pulses(rng_vals, shifts, S, obs.getFirstDM(), obs.getDMStep(),
                               obs.getNrDMs(), 20, 20.0, 2)
    best = np.unravel_index(np.argmax(grid - grid.mean(axis=1, keepdims=True)), grid.shape)
    dms = np.array([p["dm"] for p in pulses])
    ts = np.array([p["t"] for p in pulses])
    d_best = obs.getFirstDM() + best[0] * obs.getDMStep()
    k = int(np.argmin(np.abs(ts - best[1]) + np.abs(dms - d_best)))
    assert abs(dms[k] - d_best) <= 2.0 and abs(ts[k] - best[1]) <= 8


def test_float_input_against_fp64_oracle(gpu, oracle):
    """Float32 input of the same shape: bit-exact to the float restatement
    (the reference's order) and within 1e-5 relative of the FP64 oracle."""
    obs = syn.large_observation(PADDING)
    shifts = dd.getShifts(obs, PADDING)
    zapped = syn.zapped_mask(1536, 0.05, 7, PADDING)
    mapping = syn.identity_mapping(obs, PADDING)
    inp = syn.make_input(obs, 32, PADDING, seed=5, mean=128.0, sigma=20.0)
    out = syn.output_buffer(obs, dd.DD_SINGLE_STEP, PADDING)
    dd.dedispersion(obs, zapped, mapping, inp, out, shifts, PADDING, 32)
    S, row = obs.getNrSamplesPerBatch(), dd.pad(obs.getNrSamplesPerBatch(), PADDING // 4)
    rows = [0, 33, 1024, 2047]
    ref = np.zeros_like(out)
    for d in rows:
        oracle.dedispersion(obs.c, zapped, mapping, inp, ref, shifts, PADDING, 32, d, d + 1)
    got = out.reshape(-1, row)[rows, :S]
    assert np.array_equal(got.view(np.uint32), ref.reshape(-1, row)[rows, :S].view(np.uint32))
    # FP64 oracle on a prefix of DMs (the f64 entry point covers all DMs of
    # its observation): a 4-DM observation with the same channels and delays
    small = obs.copy()
    small.setDMRange(4, 0.0, obs.getDMStep())
    f64 = np.zeros((4 * row,), np.float64)
    oracle.dedispersion(small.c, zapped, mapping, inp, f64, shifts, PADDING, 32, f64=True)
    g = out.reshape(-1, row)[:4, :S].astype(np.float64)
    w = f64.reshape(-1, row)[:4, :S]
    assert (np.abs(g - w) / np.abs(w)).max() < 1e-5


def test_subband_large_matches_oracle(gpu, oracle):
    """32 subbands, 64 step-one DMs at 6.4, 32 step-two DMs at 0.2: step one
    over every sample, step two on a subset of step-one DMs."""
    obs = syn.large_observation(PADDING, subbands=True)
    shifts = dd.getShifts(obs, PADDING)
    shifts2 = dd.getShiftsStepTwo(obs, PADDING)
    zapped = syn.zapped_mask(1536, 0.05, 7, PADDING)
    inp = syn.make_input(obs, 8, PADDING, seed=3, mode=dd.DD_STEP_ONE, mean=128.0, sigma=20.0)
    mid = syn.output_buffer(obs, dd.DD_STEP_ONE, PADDING)
    dd.subbandDedispersionStepOne(obs, zapped, inp, mid, shifts, PADDING, 8)
    ref = np.zeros_like(mid)
    oracle.step_one(obs.c, zapped, inp, ref, shifts, PADDING, 8)
    assert np.array_equal(mid.view(np.uint32), ref.view(np.uint32))
    out = syn.output_buffer(obs, dd.DD_STEP_TWO, PADDING)
    lay2 = dd.layout(obs, dd.DD_STEP_TWO, 32, PADDING)
    mapping = np.zeros(lay2.mapping_row_elems, np.uint32)
    dd.subbandDedispersionStepTwo(obs, mapping, mid, out, shifts2, PADDING)
    ref2 = np.zeros_like(out)
    oracle.step_two(obs.c, mapping, mid, ref2, shifts2, PADDING)
    assert np.array_equal(out.view(np.uint32), ref2.view(np.uint32))


def test_largest_study_shape_dm_rows_match_oracle(gpu, oracle):
    """4096 channels x 8192 DMs (the top of the tuning study's range) at
    2048 samples, 5 % zapped: spread DM rows equal the oracle's."""
    obs = syn.make_observation(4096, 1220.0, 300.0 / 4096, 81.92e-6, 2048, 8192, 0.0, 0.05,
                               padding=PADDING)
    shifts = dd.getShifts(obs, PADDING)
    zapped = syn.zapped_mask(4096, 0.05, 11, PADDING)
    mapping = syn.identity_mapping(obs, PADDING)
    inp = syn.make_input(obs, 8, PADDING, seed=13, distribution="uniform")
    out = syn.output_buffer(obs, dd.DD_SINGLE_STEP, PADDING)
    dd.dedispersion(obs, zapped, mapping, inp, out, shifts, PADDING, 8)
    S, row = 2048, dd.pad(2048, PADDING // 4)
    ref = np.zeros_like(out)
    rows = [0, 1, 63, 64, 4095, 4096, 8190, 8191]
    for d in rows:
        oracle.dedispersion(obs.c, zapped, mapping, inp, ref, shifts, PADDING, 8, d, d + 1)
    got = out.reshape(-1, row)[rows, :S]
    assert np.array_equal(got.view(np.uint32), ref.reshape(-1, row)[rows, :S].view(np.uint32))
