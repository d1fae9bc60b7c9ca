"""GPU kernels against the CPU oracle, through the C ABI.

Integer inputs must match bit for bit; float input is accumulated in float32
in the reference's channel order and must match the float restatement bit for
bit too, and the FP64 oracle within a relative error of 1e-5.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn

from helpers import engine_run, oracle_run, single_case, step_one_case, step_two_case

pytestmark = pytest.mark.gpu


def assert_same(got, want, case):
    g, w = case.valid(got), case.valid(want)
    bad = np.argwhere(g.view(np.uint32) != w.view(np.uint32))
    assert bad.size == 0, (f"{len(bad)} of {g.size} samples differ; first at {bad[:5].tolist()}: "
                           f"gpu {g[tuple(bad[0])]} oracle {w[tuple(bad[0])]}")


SINGLE = [
    dict(bits=8, padding=0),                                   # unaligned rows: plain staging
    dict(bits=8, padding=64, beams=3, sbeams=5),
    dict(bits=8, padding=128, C=37, D=7, S=61, zap=0.3),
    dict(bits=8, padding=16, C=300, D=70, S=1500, zap=0.05),   # ragged time and DM tiles
    dict(bits=8, padding=16, C=520, D=33, S=700, dist="gaussian", sigma=60.0),  # > 256 rows
    dict(bits=8, padding=64, first=3.5, step=0.75, D=9),
    dict(bits=8, padding=64, zap=1.0),                         # all zapped: zeros
    dict(bits=4, padding=16, beams=2, sbeams=3),
    dict(bits=2, padding=16, C=70, D=40, S=333),
    dict(bits=1, padding=16, C=90, D=35, S=257),
    dict(bits=4, padding=0, C=33, D=5, S=77),
    dict(bits=16, padding=64, beams=2, sbeams=2, dist="gaussian", mean=1000.0, sigma=300.0),
    dict(bits=16, padding=0, C=40, D=33, S=300),
    dict(bits=32, padding=64, beams=2, sbeams=3, dist="gaussian"),
    dict(bits=32, padding=0, C=50, D=17, S=211, dist="gaussian"),
]


@pytest.mark.parametrize("kw", SINGLE)
def test_single_step_matches_oracle(gpu, oracle, kw):
    case = single_case(seed=21, **kw)
    assert_same(engine_run(case), oracle_run(oracle, case), case)


@pytest.mark.parametrize("bits,padding", [(8, 0), (8, 64), (4, 16), (2, 16), (16, 64), (32, 64)])
def test_step_one_matches_oracle(gpu, oracle, bits, padding):
    case = step_one_case(bits=bits, padding=padding, seed=13, beams=2, sdisp_multiple=8)
    assert_same(engine_run(case), oracle_run(oracle, case), case)


@pytest.mark.parametrize("padding", [0, 64])
@pytest.mark.parametrize("float_values", [False, True])
def test_step_two_matches_oracle(gpu, oracle, padding, float_values):
    case = step_two_case(padding=padding, seed=4, beams=2, sbeams=3, float_values=float_values)
    assert_same(engine_run(case), oracle_run(oracle, case), case)


def test_small_workload_bit_exact(gpu, oracle):
    """256 ch x 128 DM x 1024 samples, uint8 N(128, 16), no zapping: every sample."""
    obs = syn.small_observation(padding=128)
    shifts = dd.getShifts(obs, 128)
    z = np.zeros(256, np.uint32)
    m = syn.identity_mapping(obs, 128)
    inp = syn.make_input(obs, 8, 128, seed=1, mean=128.0, sigma=16.0)
    out = syn.output_buffer(obs, dd.DD_SINGLE_STEP, 128)
    want = np.zeros_like(out)
    dd.dedispersion(obs, z, m, inp, out, shifts, 128, 8)
    oracle.dedispersion(obs.c, z, m, inp, want, shifts, 128, 8)
    np.testing.assert_array_equal(out.view(np.uint32), want.view(np.uint32))


def test_plan_device_pointers_and_stream(gpu, oracle):
    torch = pytest.importorskip("torch")
    case = single_case(C=200, D=64, S=2048, bits=8, padding=64, zap=0.1, seed=2)
    plan = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 8, 64)
    plan.setShifts(case.shifts)
    plan.setZappedChannels(case.zapped)
    plan.setBeamMapping(case.mapping)
    d_in = torch.from_numpy(case.inp).cuda()
    d_out = torch.zeros(case.out_elems, dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    plan.run(d_in, d_out, s)
    plan.check(s)
    assert plan.launches() == 1
    assert_same(d_out.cpu().numpy(), oracle_run(oracle, case), case)
    # every compiled configuration of the family gives the same result
    for k in dd.kernels():
        if k.elem_bits != 8:
            continue
        p2 = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 8, 64, kernel=k.index)
        p2.setShifts(case.shifts)
        p2.setZappedChannels(case.zapped)
        p2.setBeamMapping(case.mapping)
        d_out.zero_()
        p2.run(d_in, d_out, s)
        p2.check(s)
        assert_same(d_out.cpu().numpy(), oracle_run(oracle, case), case)
        p2.close()
    plan.close()


@pytest.mark.parametrize("kw", [dict(C=1, D=1, S=1, bits=8), dict(C=2, D=1, S=3, bits=4),
                                dict(C=3, D=2, S=9, bits=1), dict(C=5, D=3, S=2, bits=16),
                                dict(C=1, D=4, S=5, bits=32)])
def test_degenerate_shapes_match_oracle(gpu, oracle, kw):
    """One channel, one DM, a single sample: the tile machinery at its
    smallest still equals the oracle."""
    case = single_case(padding=0, zap=0.0, seed=31, **kw)
    assert_same(engine_run(case), oracle_run(oracle, case), case)


def test_zero_dms_is_empty_work(gpu):
    """No DM trials: nothing to compute (the reference's loops run zero
    times); the call succeeds and the plan path launches nothing."""
    case = single_case(C=8, D=0, S=64, bits=8, padding=0, zap=0.0, seed=1)
    assert case.out_elems == 0
    out = np.zeros(0, np.float32)
    dd.dedispersion(case.obs, case.zapped, case.mapping, case.inp, out, case.shifts, 0, 8)
    p = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 8, 0)
    p.setShifts(case.shifts)
    p.setZappedChannels(case.zapped)
    p.setBeamMapping(case.mapping)
    torch = pytest.importorskip("torch")
    d_in = torch.from_numpy(case.inp).cuda()
    p.run(d_in, 0)
    p.check()
    p.close()


def test_every_direct_tile_in_step_one_matches_oracle(gpu, oracle):
    """Step one through every 1/2/4/8-bit direct configuration, the
    short-group tiles (groups of at most 257 rows, no 32-bit totals)
    included; and the short-group tiles refuse groups of more rows."""
    torch = pytest.importorskip("torch")
    case = step_one_case(bits=8, padding=64, seed=19, beams=2, sdisp_multiple=8)
    want = oracle_run(oracle, case)
    d_in = torch.from_numpy(case.inp).cuda()
    ran_short = 0
    for k in dd.kernels():
        if k.elem_bits != 8 or k.conf.getNrItemsD2() == 8:
            continue
        p = dd.Plan(case.obs, dd.DD_STEP_ONE, 8, 64, kernel=k.index)
        p.setShifts(case.shifts)
        p.setZappedChannels(case.zapped)
        d_out = torch.full((case.out_elems,), -1.0, dtype=torch.float32, device="cuda")
        p.run(d_in, d_out)
        p.check()
        p.close()
        assert_same(d_out.cpu().numpy(), want, case)
        ran_short += k.name.startswith("swar8s")
    assert ran_short >= 1
    big = single_case(C=300, D=8, S=256, bits=8, padding=64, zap=0.0, seed=5)  # 300 rows
    short = next(k for k in dd.kernels() if k.name.startswith("swar8s"))
    p = dd.Plan(big.obs, dd.DD_SINGLE_STEP, 8, 64, kernel=short.index)
    p.setShifts(big.shifts)
    p.setZappedChannels(big.zapped)
    p.setBeamMapping(big.mapping)
    with pytest.raises(dd.DedispersionError) as e:
        p.run(torch.from_numpy(big.inp).cuda(), torch.zeros(big.out_elems, device="cuda"))
    assert "at most 257 rows" in str(e.value)
    p.close()


def test_measured_add_rate_is_plausible(gpu):
    """dd_measure_add_rate, the roofline's denominator: float and integer add
    streams over every SM land between a quarter and 1.2x the rate of 128
    adds per SM clock at the device's maximum clock."""
    torch = pytest.importorskip("torch")
    props = torch.cuda.get_device_properties(0)
    rates = dd.measure_add_rate(0, 2)
    clock_hz = 2.2e9  # above the GB300's maximum SM clock (2.07 GHz)
    top = props.multi_processor_count * 128 * clock_hz
    for name in ("fadd_per_s", "iadd_per_s"):
        assert 0.25 * top < rates[name] < 1.2 * top, (name, rates[name], top)
