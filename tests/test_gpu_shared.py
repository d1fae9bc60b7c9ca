"""The shared-partial-sum kernels (configurations with items_d2 = 8) on the GPU.

They reach the direct sum through partial sums shared by DMs with equal
relative delays (exact integer arithmetic), so every case must equal the
oracle, and the direct kernels, bit for bit: sub-byte and 8-bit input, ragged
DM and time tiles, several beams with a mapping, unaligned rows (no bulk
copies), large DM steps (short subgroups), all-zapped, and saturated input
(every 16-bit lane at its largest before a flush).
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn
from helpers import oracle_run, single_case

pytestmark = pytest.mark.gpu


def shared_kernels():
    ks = [k for k in dd.kernels() if k.conf.getNrItemsD2() == 8]
    assert ks, "no shared-partial-sum configuration compiled"
    return ks


def run(case, kernel, torch):
    p = dd.Plan(case.obs, dd.DD_SINGLE_STEP, case.bits, case.padding, kernel=kernel)
    p.setShifts(case.shifts)
    p.setZappedChannels(case.zapped)
    p.setBeamMapping(case.mapping)
    d_in = torch.from_numpy(case.inp).cuda()
    d_out = torch.full((case.out_elems,), float("nan"), dtype=torch.float32, device="cuda")
    p.run(d_in, d_out)
    p.check()
    adds = p.adds()
    p.close()
    return d_out.cpu().numpy(), adds


def same(got, want, case):
    g = case.valid(got).view(np.uint32)
    w = case.valid(want).view(np.uint32)
    bad = np.argwhere(g != w)
    assert bad.size == 0, f"{len(bad)} mismatches, first at {bad[0]}"


@pytest.mark.parametrize("bits", [1, 2, 4, 8])
def test_ragged_tiles_every_configuration(gpu, oracle, bits):
    torch = pytest.importorskip("torch")
    case = single_case(C=256, D=100, S=1000, bits=bits, padding=128, zap=0.1, seed=bits,
                       step=0.25, dist="uniform")
    want = oracle_run(oracle, case)
    for k in shared_kernels():
        got, _ = run(case, k.index, torch)
        same(got, want, case)


def test_beams_and_mapping(gpu, oracle):
    torch = pytest.importorskip("torch")
    case = single_case(C=192, D=70, S=700, bits=8, padding=128, beams=3, sbeams=4, zap=0.2,
                       seed=4, dist="uniform")
    want = oracle_run(oracle, case)
    for k in shared_kernels():
        got, _ = run(case, k.index, torch)
        same(got, want, case)


def test_unaligned_rows_without_bulk_copies(gpu, oracle):
    torch = pytest.importorskip("torch")
    # padding 0 and an odd dispersed length: rows are not 16-byte aligned
    case = single_case(C=96, D=40, S=300, bits=8, padding=0, zap=0.1, seed=5, extra=3,
                       dist="uniform")
    assert dd.layout(case.obs, dd.DD_SINGLE_STEP, 8, 0).input_row_bytes % 16 != 0
    want = oracle_run(oracle, case)
    for k in shared_kernels():
        got, _ = run(case, k.index, torch)
        same(got, want, case)


def test_large_dm_step_cuts_subgroups(gpu, oracle):
    torch = pytest.importorskip("torch")
    # 4 MHz channels from 400 MHz: relative delays within eight channels pass
    # the limit at high DMs and subgroups shrink (to ~3.6 rows on average)
    case = single_case(C=64, D=256, S=512, bits=8, padding=128, zap=0.0, seed=6, step=0.012,
                       fmin=400.0, bw=4.0, dist="uniform")
    want = oracle_run(oracle, case)
    for k in shared_kernels():
        got, adds = run(case, k.index, torch)
        same(got, want, case)
        assert adds > 0


def test_too_large_spread_is_rejected(gpu):
    """A DM tile whose delays spread beyond the 16-bit table offsets is
    refused with DD_ERR_UNSUPPORTED-style errors at run time, not computed."""
    case = single_case(C=128, D=64, S=512, bits=8, padding=128, zap=0.0, seed=6, step=8.0,
                       fmin=300.0, bw=1.0)
    k = shared_kernels()[0]
    p = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 8, 128, kernel=k.index)
    p.setShifts(case.shifts)
    p.setZappedChannels(case.zapped)
    p.setBeamMapping(case.mapping)
    with pytest.raises(dd.DedispersionError, match="too large"):
        p.adds()
    p.close()


def test_all_zapped_is_zero(gpu):
    torch = pytest.importorskip("torch")
    case = single_case(C=64, D=32, S=256, bits=8, padding=128, zap=1.0, seed=7)
    assert (case.zapped[:64] != 0).all()
    for k in shared_kernels():
        got, adds = run(case, k.index, torch)
        assert (case.valid(got) == 0).all()
        assert adds == 0


def test_saturated_input_exact(gpu):
    """Every sample 255: each output is 255 x live channels; with 1459+ rows
    every 16-bit lane reaches 32 x 2040 before its flush."""
    torch = pytest.importorskip("torch")
    case = single_case(C=1536, D=64, S=512, bits=8, padding=128, zap=0.05, seed=8,
                       dist="constant", mean=255.0, fmin=1220.0, step=0.2, tsamp=81.92e-6)
    live = int((case.zapped[:1536] == 0).sum())
    for k in shared_kernels():
        got, _ = run(case, k.index, torch)
        assert (case.valid(got) == np.float32(255 * live)).all()


def test_full_workload_equals_direct_kernel(gpu):
    """1536 ch x 2048 DM x 24576 samples, 8-bit: the default shared plan and
    the direct kernel agree bit for bit (the direct kernel is checked against
    the oracle at this size in test_gpu_large.py), and the shared plan does
    fewer than half the adds."""
    torch = pytest.importorskip("torch")
    obs = syn.large_observation(128)
    shifts = dd.getShifts(obs, 128)
    zapped = syn.zapped_mask(1536, 0.05, 7, 128)
    mapping = syn.identity_mapping(obs, 128)
    inp = syn.make_input(obs, 8, 128, seed=1, mean=128.0, sigma=20.0, pulses=20, shifts=shifts)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, 128, shifts)
    d_in = torch.from_numpy(inp).cuda()
    outs, adds = [], []
    direct = next(k for k in dd.kernels() if k.elem_bits == 8 and k.conf.getNrItemsD2() == 1)
    for k in [direct] + shared_kernels():
        p = dd.Plan(obs, dd.DD_SINGLE_STEP, 8, 128, kernel=k.index)
        p.setShifts(shifts)
        p.setZappedChannels(zapped)
        p.setBeamMapping(mapping)
        d_out = torch.empty(lay.output_bytes // 4, dtype=torch.float32, device="cuda")
        p.run(d_in, d_out)
        p.check()
        outs.append(d_out.view(-1, lay.output_row_elems)[:, :24576].cpu().numpy())
        adds.append(p.adds())
        p.close()
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint32), outs[0].view(np.uint32))
    assert min(adds[1:]) < adds[0] / 2


@pytest.mark.parametrize("family", ["shared", "direct"])
def test_overlapped_runs_equal_serial_runs(gpu, family):
    """dd_plan_set_overlap: consecutive runs launched as programmatic
    dependents (several waves each) give the serial runs' outputs, also when
    two consecutive runs write the same output buffer; shared and direct
    tiles."""
    torch = pytest.importorskip("torch")
    want_d2 = 8 if family == "shared" else 1
    kidx = next(k.index for k in dd.kernels()
                if k.elem_bits == 8 and k.conf.getNrItemsD2() == want_d2)
    a = single_case(C=512, D=512, S=16384, bits=8, padding=128, zap=0.05, seed=41, dist="uniform")
    b = single_case(C=512, D=512, S=16384, bits=8, padding=128, zap=0.05, seed=42, dist="uniform")
    assert np.array_equal(a.shifts, b.shifts)

    def plan(overlap):
        p = dd.Plan(a.obs, dd.DD_SINGLE_STEP, 8, 128, kernel=kidx)
        p.setShifts(a.shifts)
        p.setZappedChannels(a.zapped)
        p.setBeamMapping(a.mapping)
        p.setOverlap(overlap)
        return p

    d_a, d_b = torch.from_numpy(a.inp).cuda(), torch.from_numpy(b.inp).cuda()
    new = lambda: torch.zeros(a.out_elems, dtype=torch.float32, device="cuda")
    serial = plan(False)
    want_a, want_b = new(), new()
    serial.run(d_a, want_a)
    serial.run(d_b, want_b)
    serial.check()
    ov = plan(True)
    same, out_a, out_b = new(), new(), new()
    for _ in range(5):
        ov.run(d_a, same)
        ov.run(d_b, same)      # writes what the previous launch writes
        ov.run(d_a, out_a)
        ov.run(d_b, out_b)
    ov.check()
    assert torch.equal(same, want_b) and torch.equal(out_a, want_a) and torch.equal(out_b, want_b)
    for p in (serial, ov):
        p.close()


@pytest.mark.parametrize("channels,bandwidth,step,want_shared", [
    (1536, 0.1953125, 0.2, True),     # executed adds ~0.23 of the direct sum
    (384, 0.78125, 0.467, False),     # ~0.48: the direct tile is twice as fast
])
def test_default_tile_follows_the_sharing_gain(gpu, channels, bandwidth, step, want_shared):
    """The default single-step plan keeps the shared tile only while its
    executed adds stay below 0.34 of the direct sum; either way the output is
    the direct sum (equal to the explicitly chosen other family's)."""
    torch = pytest.importorskip("torch")
    obs = syn.make_observation(channels, 1220.0, bandwidth, 81.92e-6, 4096, 1024, 0.0, step,
                               padding=128)
    shifts = dd.getShifts(obs, 128)
    zapped = syn.zapped_mask(channels, 0.05, 5, 128)
    mapping = syn.identity_mapping(obs, 128)
    d_in = syn.device_uniform_input(torch, obs, 8, 128, 9)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, 128)
    shared_idx = next(k.index for k in dd.kernels()
                      if k.elem_bits == 8 and k.conf.getNrItemsD2() == 8)
    outs, confs, adds = [], [], []
    for kidx in (None, shared_idx):
        p = dd.Plan(obs, dd.DD_SINGLE_STEP, 8, 128, kernel=kidx)
        p.setShifts(shifts)
        p.setZappedChannels(zapped)
        p.setBeamMapping(mapping)
        d_out = torch.zeros(lay.output_bytes // 4, dtype=torch.float32, device="cuda")
        p.run(d_in, d_out)
        p.check()
        outs.append(d_out.cpu().numpy())
        confs.append(p.conf())
        adds.append(p.adds())
        p.close()
    live = int((np.asarray(zapped)[:channels] == 0).sum())
    ratio = adds[1] / (live * 1024 * obs.getNrSamplesPerBatch())
    assert (ratio < 0.34) == want_shared, ratio
    assert (confs[0].getNrItemsD2() == 8) == want_shared
    np.testing.assert_array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))


def test_table_change_while_a_run_is_in_flight(gpu, oracle):
    """A setter called right after a run was enqueued on a non-blocking
    stream: the next use rebuilds the tables and waits for the device before
    it uploads them, so the run in flight reads the old tables to the end
    (its output equals the oracle's for the old mask) and the next run uses
    the new ones."""
    torch = pytest.importorskip("torch")
    case = single_case(C=1024, D=512, S=8192, bits=8, padding=128, zap=0.05, seed=61,
                       fmin=1220.0, tsamp=81.92e-6, step=0.2)
    new_zapped = case.zapped.copy()
    new_zapped[:case.obs.getNrChannels() // 2] = 1          # zap half the band
    plan = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 8, case.padding)
    plan.setShifts(case.shifts)
    plan.setZappedChannels(case.zapped)
    plan.setBeamMapping(case.mapping)
    d_in = torch.from_numpy(case.inp).cuda()
    out1 = torch.zeros(case.out_elems, dtype=torch.float32, device="cuda")
    out2 = torch.zeros_like(out1)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # the input copy and the fills
    plan.run(d_in, out1, s)                 # in flight ...
    plan.setZappedChannels(new_zapped)      # ... while the mask changes
    plan.run(d_in, out2, s)
    plan.check(s)
    plan.close()
    want1 = oracle_run(oracle, case)
    case2 = single_case(C=1024, D=512, S=8192, bits=8, padding=128, zap=0.05, seed=61,
                        fmin=1220.0, tsamp=81.92e-6, step=0.2)
    case2.zapped[:] = new_zapped
    want2 = oracle_run(oracle, case2)
    same(out1.cpu().numpy(), want1, case)
    same(out2.cpu().numpy(), want2, case2)


def test_default_direct_tile_keeps_two_ctas_worth_of_warps(gpu, oracle):
    """384 channels of 8-bit input at a DM step of 0.46: the shared tile is
    not worth it, and the 8-warp direct tile's staged window (a wide DM
    spread) leaves room for one CTA per SM; the default then takes the
    16-warp tile of the same shape, with the oracle's output."""
    torch = pytest.importorskip("torch")
    case = single_case(C=384, D=256, S=4096, bits=8, padding=128, zap=0.05, seed=67,
                       fmin=1220.0, bw=0.78125, tsamp=81.92e-6, step=0.459)
    p = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 8, 128)
    p.setShifts(case.shifts)
    p.setZappedChannels(case.zapped)
    p.setBeamMapping(case.mapping)
    d_out = torch.zeros(case.out_elems, dtype=torch.float32, device="cuda")
    p.run(torch.from_numpy(case.inp).cuda(), d_out)
    p.check()
    conf = p.conf()
    p.close()
    assert conf.getNrItemsD2() == 1 and conf.getNrThreadsD1() == 16, conf.print()
    same(d_out.cpu().numpy(), oracle_run(oracle, case), case)
