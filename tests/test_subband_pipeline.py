"""Subband pipeline (dd_subband_*): step one then step two on the device.

The output must equal the oracle's step one followed by its step two
(include/Dedispersion.hpp:111-176) bit for bit: with the packed 16-bit
intermediate (1-8-bit input whose subband sums fit 16 bits: odd and even
coarse-DM counts, lane widening every few subbands, saturated input) and
with the float intermediate it falls back to (16-bit input, wide subbands).
At the full 1536-channel, 32-subband shape the packed pipeline equals the
oracle chain and the engine's own two float steps.  The subband frequencies
of step two (getShiftsStepTwo) follow AstroData's subband accessors, which
the reference's sources do not include: the oracle restates them
(oracle/dd_oracle.c), so step two is pinned to the restatement, not to
AstroData itself.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn
from helpers import subband_obs

pytestmark = pytest.mark.gpu


def _case(bits=8, padding=0, seed=0, zap=0.1, sbeams=3, beams=2, fill=None, **kw):
    obs = subband_obs(padding=padding, beams=beams, sbeams=sbeams, **kw)
    shifts = dd.getShifts(obs, padding)
    shifts2 = dd.getShiftsStepTwo(obs, padding)
    zapped = syn.zapped_mask(obs.getNrChannels(), zap, seed + 7, padding)
    inp = syn.make_input(obs, bits, padding, seed, mode=dd.DD_STEP_ONE)
    if fill is not None:
        inp[:] = fill
    l2 = dd.layout(obs, dd.DD_STEP_TWO, 32, padding)
    rng = np.random.default_rng(seed + 5)
    mapping = np.zeros((sbeams, l2.mapping_row_elems), np.uint32)
    mapping[:, :obs.getNrSubbands()] = rng.integers(0, beams, size=(sbeams, obs.getNrSubbands()))
    return obs, shifts, shifts2, zapped, inp, mapping.reshape(-1)


def _oracle_chain(oracle, obs, shifts, shifts2, zapped, inp, mapping, padding, bits):
    l1 = dd.layout(obs, dd.DD_STEP_ONE, bits, padding)
    l2 = dd.layout(obs, dd.DD_STEP_TWO, 32, padding)
    inter = np.zeros(l1.output_bytes // 4, np.float32)
    oracle.step_one(obs.c, zapped, inp, inter, shifts, padding, bits)
    out = np.zeros(l2.output_bytes // 4, np.float32)
    oracle.step_two(obs.c, mapping, inter, out, shifts2, padding)
    return out


def _pipeline(obs, shifts, shifts2, zapped, inp, mapping, padding, bits, pair_kernel=0,
              chunks=0):
    torch = pytest.importorskip("torch")
    p = dd.SubbandPipeline(obs, bits, padding)
    if pair_kernel:
        p.setPairKernel(pair_kernel)
    if chunks:
        p.setChunks(chunks)
    p.setTables(shifts, shifts2, zapped, mapping)
    d_in = torch.from_numpy(np.ascontiguousarray(inp).view(np.uint8).reshape(-1)).cuda()
    d_out = torch.zeros(p.layout_out.output_bytes // 4, dtype=torch.float32, device="cuda")
    p.run(d_in, d_out)
    p.check()
    info = p.info()
    p.close()
    return d_out.cpu().numpy(), info


CASES = [
    dict(bits=8, padding=0, D1=8),
    dict(bits=8, padding=64, D1=7),                  # odd: the last pair has one coarse DM
    dict(bits=4, padding=16, D1=6),
    dict(bits=2, padding=16, D1=5),
    dict(bits=1, padding=0, D1=4),
    dict(bits=8, padding=64, D1=9, C=512, SB=4),    # 128 ch per subband: widen every 2 rows
    dict(bits=4, padding=64, D1=6, C=600, SB=2, zap=0.0),  # 300 rows per subband: the step-one
                                                            # tile with 32-bit totals
]


@pytest.mark.parametrize("kw", CASES)
def test_packed_pipeline_matches_oracle_chain(gpu, oracle, kw):
    kw = dict(kw)
    bits, padding = kw.pop("bits"), kw.pop("padding")
    args = _case(bits=bits, padding=padding, seed=3, **kw)
    want = _oracle_chain(oracle, *args, padding, bits)
    got, info = _pipeline(*args, padding, bits)
    assert info["packed"]
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("bits,chunks,kw", [
    (8, 2, dict(D1=7, S=1500)),
    (8, 5, dict(D1=8, S=2100, D2=20)),
    (4, 3, dict(D1=6, S=1300)),
    (8, 200, dict(D1=5, S=1100)),              # more chunks than time tiles
    (16, 4, dict(D1=5, S=1700)),               # float intermediate
])
def test_chunked_pipeline_matches_oracle_chain(gpu, oracle, bits, chunks, kw):
    """dd_subband_set_chunks: step two in time ranges, each right after the
    step-one tiles it reads (step one on the pipeline's side stream)."""
    args = _case(bits=bits, padding=64, seed=13, **kw)
    want = _oracle_chain(oracle, *args, 64, bits)
    got, info = _pipeline(*args, 64, bits, chunks=chunks)
    assert info["packed"] == (bits <= 8)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_every_pair_tile_matches(gpu, oracle):
    args = _case(bits=8, padding=64, seed=11, D1=7, D2=24, S=300)
    want = _oracle_chain(oracle, *args, 64, 8)
    for k in range(dd.pair_kernel_count()):
        got, info = _pipeline(*args, 64, 8, pair_kernel=k)
        assert info["packed"]
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=str(k))


def test_saturated_input_widens_lanes(gpu, oracle):
    """Every sample 255 with 128 live channels per subband: each step-one sum
    is 32640, the four-subband total 130560, past the 16-bit lanes."""
    args = _case(bits=8, padding=64, seed=2, zap=0.0, D1=4, C=512, SB=4, fill=255)
    want = _oracle_chain(oracle, *args, 64, 8)
    got, info = _pipeline(*args, 64, 8)
    assert info["packed"] and want.max() == 4 * 128 * 255
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("bits,kw", [(16, dict(D1=5)), (8, dict(D1=4, C=600, SB=2))])
def test_float_intermediate_when_sums_can_exceed_16_bits(gpu, oracle, bits, kw):
    args = _case(bits=bits, padding=64, seed=5, **kw)
    want = _oracle_chain(oracle, *args, 64, bits)
    got, info = _pipeline(*args, 64, bits)
    assert not info["packed"]
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_host_call_matches_oracle_chain(gpu, oracle):
    """The host-buffer call, three times: its cached pipeline is reused, then
    rebuilt when the zapped mask changes."""
    obs, shifts, shifts2, zapped, inp, mapping = _case(bits=8, padding=64, seed=8, D1=6)
    row = dd.layout(obs, dd.DD_STEP_TWO, 32, 64).output_row_elems
    S = obs.getNrSamplesPerBatch()
    zapped2 = zapped.copy()
    zapped2[:7] = 1
    for z in (zapped, zapped, zapped2):
        want = _oracle_chain(oracle, obs, shifts, shifts2, z, inp, mapping, 64, 8)
        out = np.full(dd.layout(obs, dd.DD_STEP_TWO, 32, 64).output_bytes // 4, -1.0, np.float32)
        dd.subbandDedispersion(obs, z, mapping, inp, out, shifts, shifts2, 64, 8)
        np.testing.assert_array_equal(out.reshape(-1, row)[:, :S], want.reshape(-1, row)[:, :S])


def test_full_shape_equals_float_steps(gpu, oracle):
    """1536 channels (5 % zapped), 32 subbands, 64 x 32 DMs, 24576 samples:
    the packed pipeline equals the oracle's step one + step two and the
    engine's float step one + step two."""
    torch = pytest.importorskip("torch")
    obs = syn.large_observation(128, subbands=True)
    shifts, shifts2 = dd.getShifts(obs, 128), dd.getShiftsStepTwo(obs, 128)
    zapped = syn.zapped_mask(1536, 0.05, 7, 128)
    mapping = syn.identity_mapping(obs, 128, subbands=True)
    l1 = dd.layout(obs, dd.DD_STEP_ONE, 8, 128)
    l2 = dd.layout(obs, dd.DD_STEP_TWO, 32, 128)
    g = torch.Generator(device="cuda")
    g.manual_seed(12)
    d_in = torch.randint(0, 256, (l1.input_bytes,), generator=g, dtype=torch.uint8, device="cuda")
    p = dd.SubbandPipeline(obs, 8, 128)
    p.setTables(shifts, shifts2, zapped, mapping)
    assert p.info()["packed"]
    got = torch.zeros(l2.output_bytes // 4, dtype=torch.float32, device="cuda")
    p.run(d_in, got)
    p.check()
    one = dd.Plan(obs, dd.DD_STEP_ONE, 8, 128)
    one.setShifts(shifts)
    one.setZappedChannels(zapped)
    two = dd.Plan(obs, dd.DD_STEP_TWO, 32, 128)
    two.setShifts(shifts2)
    two.setBeamMapping(mapping)
    inter = torch.zeros(l1.output_bytes // 4, dtype=torch.float32, device="cuda")
    want = torch.zeros_like(got)
    one.run(d_in, inter)
    two.run(inter, want)
    two.check()
    assert torch.equal(got, want)
    ref = _oracle_chain(oracle, obs, shifts, shifts2, zapped, d_in.cpu().numpy(), mapping, 128, 8)
    assert np.array_equal(got.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    # chunked runs, twice back to back (the second run's step one waits for
    # the first run's step two)
    p.setChunks(6)
    for _ in range(2):
        got.zero_()
        p.run(d_in, got)
    p.check()
    assert torch.equal(got, want)
    for x in (p, one, two):
        x.close()


def test_overlapped_pipeline_runs_equal_serial_runs(gpu):
    """dd_subband_set_overlap: step one of each run starts while the
    previous run's step two finishes; outputs equal serial runs."""
    torch = pytest.importorskip("torch")
    obs, shifts, shifts2, zapped, inp_a, mapping = _case(bits=8, padding=64, seed=21, D1=16,
                                                           D2=32, S=4096, C=512, SB=16)
    inp_b = syn.make_input(obs, 8, 64, 22, mode=dd.DD_STEP_ONE)

    def pipe(overlap):
        p = dd.SubbandPipeline(obs, 8, 64)
        p.setTables(shifts, shifts2, zapped, mapping)
        p.setOverlap(overlap)
        return p

    d_a, d_b = torch.from_numpy(inp_a).cuda(), torch.from_numpy(inp_b).cuda()
    serial, ov = pipe(False), pipe(True)
    new = lambda: torch.zeros(serial.layout_out.output_bytes // 4, dtype=torch.float32,
                              device="cuda")
    want_a, want_b = new(), new()
    serial.run(d_a, want_a)
    serial.run(d_b, want_b)
    serial.check()
    out_a, out_b = new(), new()
    for _ in range(4):
        ov.run(d_a, out_a)
        ov.run(d_b, out_b)
    ov.check()
    assert torch.equal(out_a, want_a) and torch.equal(out_b, want_b)
    serial.close()
    ov.close()
