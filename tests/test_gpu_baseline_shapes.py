"""Oracle parity at the real shapes of the measured workloads.

* 40 uneven beams in one batch (384/1536 channels, 8192-32768 samples,
  512-4096 DMs at 0.1-0.5, 2/4/8-bit uniform input, 5 % zapped): every beam
  equals the plain path sample for sample in both batch forms (concurrent
  graph branches and the persistent kernel), and every beam equals the CPU
  oracle (include/Dedispersion.hpp:70-109) on a spread of DM rows that
  includes DM-tile edges.
* 12 served beams (1536 channels, 25000-sample 8-bit batches, 1024-4096 DMs
  at 0.2, single-step and 32-subband streams): two consecutive batches per
  beam, each equal to the oracle on its window [carried tail | batch] --
  single-step beams on a spread of DM rows, subband beams on every row of the
  oracle's step one followed by its step two
  (include/Dedispersion.hpp:111-176).

The subband frequencies the step-two shifts use (AstroData's
getSubbandMinFreq/MaxFreq, not in the reference tree) cannot be pinned
against the reference: the engine and the oracle share one definition, the
frequency of a subband's highest channel.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import serving
from dedispersion_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

PADDING = 128


def spread_rows(D, rng, extra=6):
    edges = [0, 1, 31, 32, 33, 63, 64, 65, 127, 128, D // 2, D - 65, D - 64, D - 33, D - 32,
             D - 2, D - 1]
    rand = rng.integers(0, D, size=extra).tolist()
    return sorted({int(r) for r in edges + rand if 0 <= r < D})


@pytest.fixture(scope="module")
def batched(gpu):
    torch = pytest.importorskip("torch")
    beams = []
    for sh in syn.batched_shapes(40):
        obs = syn.shape_observation(sh, PADDING)
        shifts = dd.getShifts(obs, PADDING)
        zapped = syn.zapped_mask(sh["channels"], 0.05, sh["seed"], PADDING)
        mapping = syn.identity_mapping(obs, PADDING)
        d_in = syn.device_uniform_input(torch, obs, sh["bits"], PADDING, sh["seed"])
        lay = dd.layout(obs, dd.DD_SINGLE_STEP, sh["bits"], PADDING)
        beams.append(dict(sh=sh, obs=obs, shifts=shifts, zapped=zapped, mapping=mapping,
                          d_in=d_in, lay=lay))
    yield torch, beams
    torch.cuda.empty_cache()


def _valid(t, lay, S):
    rows = lay.output_bytes // 4 // lay.output_row_elems
    return t.view(rows, -1)[:, :S]


def test_batched_40_beams_equal_plain_and_oracle(batched, oracle):
    torch, beams = batched
    # plain path, one beam at a time
    plain = []
    for b in beams:
        plan = dd.Plan(b["obs"], dd.DD_SINGLE_STEP, b["sh"]["bits"], PADDING)
        plan.setShifts(b["shifts"])
        plan.setZappedChannels(b["zapped"])
        plan.setBeamMapping(b["mapping"])
        out = torch.empty(b["lay"].output_bytes // 4, dtype=torch.float32, device="cuda")
        plan.run(b["d_in"], out)
        plan.check()
        plan.close()
        plain.append(out)
    rng = np.random.default_rng(40)
    for i, b in enumerate(beams):
        S, D = b["obs"].getNrSamplesPerBatch(), b["obs"].getNrDMs()
        rows = spread_rows(D, rng)
        ref = np.zeros(b["lay"].output_bytes // 4, np.float32)
        host_in = b["d_in"].cpu().numpy()
        for d in rows:
            oracle.dedispersion(b["obs"].c, b["zapped"], b["mapping"], host_in, ref, b["shifts"],
                                PADDING, b["sh"]["bits"], d, d + 1)
        want = ref.reshape(-1, b["lay"].output_row_elems)[rows, :S]
        got = _valid(plain[i], b["lay"], S)[rows].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (i, b["sh"])
    # both batch forms, beam by beam against the plain outputs
    for persistent in (False, True):
        batch = dd.Batch()
        outs = []
        for b in beams:
            out = torch.full((b["lay"].output_bytes // 4,), -1.0, device="cuda")
            batch.add(b["obs"], b["sh"]["bits"], PADDING, b["shifts"], b["zapped"], b["mapping"],
                      b["d_in"], out)
            outs.append(out)
        if persistent:
            batch.setPersistent(True)
        batch.commit()
        assert batch.info()["form"] == ("persistent" if persistent else "graph")
        for _ in range(2):  # two replays of the recorded graph
            for o in outs:
                o.fill_(-1.0)
            batch.run()
            batch.check()
            for i, b in enumerate(beams):
                S = b["obs"].getNrSamplesPerBatch()
                assert torch.equal(_valid(outs[i], b["lay"], S), _valid(plain[i], b["lay"], S)), \
                    (persistent, i, b["sh"])
        batch.close()
        del outs
    torch.cuda.synchronize()


def _window_obs(stream, window_samples):
    obs = stream.obs.copy()
    obs.setNrSamplesPerDispersedBatch(window_samples)
    return obs


def _oracle_single(oracle, stream, window, rows):
    cfg = stream.cfg
    obs = _window_obs(stream, window.shape[1])
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, cfg.bits, cfg.padding)
    inp = np.zeros((cfg.channels, lay.input_row_bytes), np.uint8)
    inp[:, :window.shape[1]] = window
    out = np.zeros(lay.output_bytes // 4, np.float32)
    mapping = np.zeros(lay.mapping_row_elems, np.uint32)
    for d in rows:
        oracle.dedispersion(obs.c, stream.zapped, mapping, inp.reshape(-1), out, stream.shifts,
                            cfg.padding, cfg.bits, d, d + 1)
    return out.reshape(-1, lay.output_row_elems)[rows, :cfg.samples]


def _oracle_subband(oracle, stream, window):
    cfg = stream.cfg
    obs = stream.obs.copy()
    tail2 = dd.layout(stream.obs, dd.DD_STEP_TWO, 32, cfg.padding, stream.shifts2).max_delay
    obs.setNrSamplesPerBatch(cfg.samples + tail2, True)
    obs.setNrSamplesPerDispersedBatch(window.shape[1], True)
    lay1 = dd.layout(obs, dd.DD_STEP_ONE, cfg.bits, cfg.padding)
    inp = np.zeros((cfg.channels, lay1.input_row_bytes), np.uint8)
    inp[:, :window.shape[1]] = window
    mid = np.zeros(lay1.output_bytes // 4, np.float32)
    oracle.step_one(obs.c, stream.zapped, inp.reshape(-1), mid, stream.shifts, cfg.padding,
                    cfg.bits)
    lay2 = dd.layout(obs, dd.DD_STEP_TWO, 32, cfg.padding)
    out = np.zeros(lay2.output_bytes // 4, np.float32)
    oracle.step_two(obs.c, np.zeros(lay2.mapping_row_elems, np.uint32), mid, out,
                    stream.shifts2, cfg.padding)
    return out.reshape(-1, lay2.output_row_elems)[:, :cfg.samples]


def test_served_12_beams_two_batches_equal_oracle(gpu, oracle):
    pytest.importorskip("torch")
    cfgs = serving.served_beams(12, seed=77, padding=PADDING, double_buffer=True)
    server = serving.Server(budget_bytes=150 * 10**9)
    for c in cfgs:
        server.admit(c)
    nb = 2
    data = {}
    outputs = {}

    def source(b, k, staging):
        g = np.random.default_rng(1000 * cfgs[b].seed + k)
        data[(b, k)] = g.integers(0, 256, size=(cfgs[b].channels, cfgs[b].samples),
                                  dtype=np.uint8)
        staging[:, :cfgs[b].samples] = data[(b, k)]

    def consumer(b, k, out):
        outputs[(b, k)] = out.copy()

    sched = [(0.0, b, k) for k in range(nb) for b in range(len(cfgs))]
    report = server.serve(sched, source, consumer, deadline=cfgs[0].period)
    assert report.summary()["batches"] == nb * len(cfgs)
    rng = np.random.default_rng(5)
    for b, stream in enumerate(server.streams):
        cfg = stream.cfg
        assert stream.output_rows == cfg.dms
        prev = np.zeros((cfg.channels, stream.tail), np.uint8)
        for k in range(nb):
            window = np.concatenate([prev, data[(b, k)]], axis=1)
            got = outputs[(b, k)]
            if cfg.subband:
                want = _oracle_subband(oracle, stream, window)
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (cfg.name, k)
            else:
                rows = spread_rows(cfg.dms, rng)
                want = _oracle_single(oracle, stream, window, rows)
                assert np.array_equal(got[rows].view(np.uint32), want.view(np.uint32)), \
                    (cfg.name, k)
            prev = window[:, window.shape[1] - stream.tail:]
            data.pop((b, k))
            outputs.pop((b, k))
    server.close()


def test_served_admission_at_the_12_beam_shape(gpu):
    """A budget that holds only part of the 12 beams: beams are admitted in
    order while their device bytes fit, the others are refused with
    DD_ERR_OVER_BUDGET and leave nothing allocated."""
    cfgs = serving.served_beams(12, seed=77, padding=PADDING, double_buffer=True)
    need = [serving.stream_bytes(c)[0] for c in cfgs]
    budget = sum(need[:5]) + need[5] // 2
    server = serving.Server(budget_bytes=budget)
    admitted, refused = [], []
    for i, c in enumerate(cfgs):
        try:
            server.admit(c)
            admitted.append(i)
        except dd.DedispersionError as e:
            assert e.status == dd._abi.DD_ERR_OVER_BUDGET
            refused.append(i)
    used = 0
    expect = []
    for i, n in enumerate(need):
        if used + n <= budget:
            used += n
            expect.append(i)
    assert admitted == expect and len(admitted) < 12 and refused
    assert server.used == sum(need[i] for i in admitted) <= budget
    server.close()
