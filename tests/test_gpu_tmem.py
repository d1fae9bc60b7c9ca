"""The TMEM-window tile (float32 single step) against the oracle and the
scalar tile.

The tile keeps each thread's window of input samples in tensor memory and
reads one DM's 16 samples with one tcgen05.ld; rows are summed in the
reference's channel order (include/Dedispersion.hpp:79-104), so its output
must equal the float restatement, and the scalar tile, bit for bit.  Shapes
whose 16-DM delay spread does not fit its 48-sample windows fall back to the
scalar tile.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd

from helpers import oracle_run, single_case

pytestmark = pytest.mark.gpu

TMEM = "tmem32_t16_d64"
SCALAR = "scalar32_i8_d8_w4_c16"


def _kernel(name):
    return next(k.index for k in dd.kernels() if k.name == name)


def _run(case, kernel=None, offset=0):
    """One plan run on device buffers; `offset` floats shift the input's start
    (an offset of 1 leaves it 4-byte aligned only: the tile's plain-load path)."""
    torch = pytest.importorskip("torch")
    plan = dd.Plan(case.obs, dd.DD_SINGLE_STEP, 32, case.padding,
                   kernel=None if kernel is None else _kernel(kernel))
    plan.setShifts(case.shifts)
    plan.setZappedChannels(case.zapped)
    plan.setBeamMapping(case.mapping)
    flat = torch.from_numpy(case.inp.view(np.float32).reshape(-1))
    buf = torch.zeros(flat.numel() + offset, dtype=torch.float32, device="cuda")
    buf[offset:] = flat.cuda()
    d_in = buf[offset:]
    d_out = torch.full((case.out_elems,), -1.0, dtype=torch.float32, device="cuda")
    plan.run(d_in, d_out)
    plan.check()
    d2 = plan.conf().getNrItemsD2()
    plan.close()
    return d_out.cpu().numpy(), d2


def _same(got, want, case):
    g, w = case.valid(got), case.valid(want)
    bad = np.argwhere(g.view(np.uint32) != w.view(np.uint32))
    assert bad.size == 0, f"{len(bad)} of {g.size} samples differ; first at {bad[:3].tolist()}"


CASES = [
    dict(C=1536, D=130, S=2000, padding=128, fmin=1220.0, tsamp=81.92e-6, step=0.2),
    dict(C=50, D=17, S=211, padding=64),                   # ragged: rows, DMs, samples
    dict(C=256, D=200, S=1100, padding=64, beams=2, sbeams=3),  # mapped beams
    dict(C=300, D=70, S=1500, padding=16, zap=0.3),
    dict(C=64, D=64, S=512, padding=64, zap=1.0),          # all zapped: zeros
]


@pytest.mark.parametrize("kw", CASES, ids=[f"C{c['C']}_D{c['D']}_S{c['S']}" for c in CASES])
def test_default_float_plan_runs_tmem_tile_bit_exact(gpu, oracle, kw):
    case = single_case(bits=32, dist="gaussian", seed=31, **kw)
    got, d2 = _run(case)
    assert d2 == 3, "plans without a configuration run the TMEM-window tile on float input"
    _same(got, oracle_run(oracle, case), case)


def test_unaligned_input_takes_plain_loads(gpu, oracle):
    case = single_case(bits=32, C=200, D=90, S=900, padding=64, dist="gaussian", seed=33)
    got, d2 = _run(case, kernel=TMEM, offset=1)
    assert d2 == 3
    _same(got, oracle_run(oracle, case), case)


def test_equals_scalar_tile(gpu):
    case = single_case(bits=32, C=1024, D=256, S=4096, padding=128, fmin=1220.0,
                       tsamp=81.92e-6, step=0.2, dist="gaussian", seed=35, zap=0.05)
    a, _ = _run(case, kernel=TMEM)
    b, _ = _run(case, kernel=SCALAR)
    _same(a, b, case)


def test_wide_spread_falls_back_to_scalar(gpu, oracle):
    # 16 DMs at step 4 move the lowest channel's delay by far more than 48
    # samples: the default plan takes the scalar tile; the TMEM tile refuses.
    case = single_case(bits=32, C=128, D=40, S=600, padding=64, step=4.0, dist="gaussian",
                       seed=37)
    got, d2 = _run(case)
    assert d2 == 1
    _same(got, oracle_run(oracle, case), case)
    with pytest.raises(dd.DedispersionError) as e:
        _run(case, kernel=TMEM)
    assert "16 DMs spread a row's delay" in str(e.value)


def test_full_size_float_rows(gpu, oracle):
    """The 1536 ch x 2048 DM x 24576-sample workload with float32 input
    (N(128, 20), 5 % zapped): every DM row equals the scalar tile's bit for
    bit, and 64 DM rows spread over the range equal the oracle's."""
    torch = pytest.importorskip("torch")
    from dedispersion_gb300 import synthetic as syn
    obs = syn.large_observation(128)
    shifts = dd.getShifts(obs, 128)
    zapped = syn.zapped_mask(1536, 0.05, 7, 128)
    mapping = syn.identity_mapping(obs, 128)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 32, 128)
    rng = np.random.default_rng(41)
    row = lay.input_row_bytes // 4
    inp = np.zeros((1536, row), np.float32)
    n = obs.getNrSamplesPerDispersedBatch()
    inp[:, :n] = rng.normal(128.0, 20.0, size=(1536, n)).astype(np.float32)
    d_in = torch.from_numpy(inp).cuda()
    outs = {}
    for name in (TMEM, SCALAR):
        p = dd.Plan(obs, dd.DD_SINGLE_STEP, 32, 128, kernel=_kernel(name))
        p.setShifts(shifts)
        p.setZappedChannels(zapped)
        p.setBeamMapping(mapping)
        d_out = torch.full((lay.output_bytes // 4,), -1.0, dtype=torch.float32, device="cuda")
        p.run(d_in, d_out)
        p.check()
        p.close()
        outs[name] = d_out.cpu().numpy()
    D, S = obs.getNrDMs(), obs.getNrSamplesPerBatch()
    a = outs[TMEM].reshape(D, -1)[:, :S]
    b = outs[SCALAR].reshape(D, -1)[:, :S]
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    want = np.zeros(lay.output_bytes // 4, np.float32)
    for d in np.linspace(0, D - 1, 64).astype(int):
        oracle.dedispersion(obs.c, zapped, mapping, inp, want, shifts, 128, 32,
                            dm_begin=int(d), dm_end=int(d) + 1)
        w = want.reshape(D, -1)[d, :S]
        assert np.array_equal(a[d].view(np.uint32), w.view(np.uint32)), f"DM row {d}"
