"""Detection statistics of the output (dd_plan_run_stats, dd_dm_stats_from_accum).

Per output row: the exact integer sum, sum of squares and earliest largest
sample, accumulated in the shared-partial-sum kernel's epilogue or by a pass
over the output for the other kernels; both must equal numpy's on the output
the same call wrote, and the S/N peak must sit at an injected pulse.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn
from helpers import single_case


def test_stats_from_accumulators():
    # rows: [1, 2, 3, 4] -> sum 10, sum_sq 30, peak 4 at sample 3; constant row
    acc = np.array([[10, 30, (4 << 32) | (0xFFFFFFFF - 3)],
                    [20, 100, (5 << 32) | (0xFFFFFFFF - 0)]], np.uint64)
    st = dd.dm_stats(acc, 4)
    assert st["mean"][0] == 2.5 and st["stddev"][0] == pytest.approx(np.std([1, 2, 3, 4]))
    assert st["peak"][0] == 4 and st["peak_sample"][0] == 3
    assert st["snr"][0] == pytest.approx(1.5 / np.std([1, 2, 3, 4]))
    assert st["stddev"][1] == 0 and st["snr"][1] == 0 and st["peak_sample"][1] == 0


def _expect(out, rows, S, row_len):
    grid = out.reshape(rows, row_len)[:, :S].astype(np.uint64)
    s1 = grid.sum(axis=1)
    s2 = (grid * grid).sum(axis=1)
    peak = grid.max(axis=1)
    first = grid.argmax(axis=1).astype(np.uint64)
    key = (peak << np.uint64(32)) | (np.uint64(0xFFFFFFFF) - first)
    return np.stack([s1, s2, key], axis=1)


@pytest.mark.gpu
@pytest.mark.parametrize("family", ["shared", "direct"])
@pytest.mark.parametrize("bits", [2, 8])
def test_accumulators_match_output(gpu, family, bits):
    torch = pytest.importorskip("torch")
    case = single_case(C=256, D=100, S=1000, bits=bits, padding=128, sbeams=2, beams=2,
                       zap=0.1, seed=3, dist="uniform")
    want_d2 = 8 if family == "shared" else 1
    k = next(k for k in dd.kernels() if k.elem_bits == 8 and k.conf.getNrItemsD2() == want_d2)
    p = dd.Plan(case.obs, dd.DD_SINGLE_STEP, bits, 128, kernel=k.index)
    p.setShifts(case.shifts)
    p.setZappedChannels(case.zapped)
    p.setBeamMapping(case.mapping)
    d_in = torch.from_numpy(case.inp).cuda()
    d_out = torch.zeros(case.out_elems, dtype=torch.float32, device="cuda")
    rows = case.out_rows
    d_acc = torch.full((rows, 3), 7, dtype=torch.int64, device="cuda")  # cleared by the call
    for _ in range(2):
        p.run_stats(d_in, d_out, d_acc)
        p.check()
    out = d_out.cpu().numpy()
    got = d_acc.cpu().numpy().view(np.uint64)
    want = _expect(out, rows, case.nr_samples, case.out_row)
    np.testing.assert_array_equal(got, want)
    st = dd.dm_stats(got, case.nr_samples)
    grid = out.reshape(rows, case.out_row)[:, :case.nr_samples].astype(np.float64)
    np.testing.assert_allclose(st["mean"], grid.mean(axis=1), rtol=1e-12)
    np.testing.assert_allclose(st["stddev"], grid.std(axis=1), rtol=1e-9)
    p.close()


@pytest.mark.gpu
def test_pulse_is_the_snr_peak(gpu):
    """1536 channels x 256 DMs with one bright dispersed pulse: the largest
    S/N over all DMs is within a few DMs and samples of it."""
    torch = pytest.importorskip("torch")
    obs = syn.make_observation(1536, 1220.0, 0.1953125, 81.92e-6, 4096, 256, 0.0, 0.2,
                               padding=128)
    shifts = dd.getShifts(obs, 128)
    zapped = syn.zapped_mask(1536, 0.05, 7, 128)
    mapping = syn.identity_mapping(obs, 128)
    inp = syn.make_input(obs, 8, 128, seed=9, mean=128.0, sigma=20.0, pulses=1, shifts=shifts)
    pulses = syn.inject_pulses(np.zeros((1, 1536, obs.getNrSamplesPerDispersedBatch()), np.uint8),
                               shifts, 4096, 0.0, 0.2, 256, 1, 20.0, 10)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, 128, shifts)
    p = dd.Plan(obs, dd.DD_SINGLE_STEP, 8, 128)
    p.setShifts(shifts)
    p.setZappedChannels(zapped)
    p.setBeamMapping(mapping)
    d_in = torch.from_numpy(inp).cuda()
    d_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32, device="cuda")
    d_acc = torch.empty((256, 3), dtype=torch.int64, device="cuda")
    p.run_stats(d_in, d_out, d_acc)
    p.check()
    st = dd.dm_stats(d_acc.cpu().numpy().view(np.uint64), 4096)
    best = int(np.argmax(st["snr"]))
    assert abs(0.2 * best - pulses[0]["dm"]) <= 1.0
    assert abs(int(st["peak_sample"][best]) - pulses[0]["t"]) <= 8
    assert st["snr"][best] > 6
    p.close()


@pytest.mark.gpu
def test_float_input_is_rejected(gpu):
    case = single_case(C=32, D=8, S=64, bits=32, padding=128)
    p = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 32, 128)
    p.setShifts(case.shifts)
    p.setZappedChannels(case.zapped)
    p.setBeamMapping(case.mapping)
    with pytest.raises(dd.DedispersionError, match="1-16 bits"):
        p.run_stats(1, 1, 1)
    p.close()
