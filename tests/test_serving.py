"""Real-time serving: admission by device-memory budget, and every served
batch equal to the oracle (include/Dedispersion.hpp:70-176) on its window
[tail | batch]."""
import dataclasses

import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import _abi, serving
from dedispersion_gb300 import synthetic as syn


def small_beams():
    return [
        serving.BeamConfig(name="single8", channels=256, bandwidth=0.5, samples=4096, dms=128,
                           dm_step=0.2, bits=8, seed=1),
        serving.BeamConfig(name="subband8", channels=256, bandwidth=0.5, samples=4096, dms=128,
                           dm_step=0.2, bits=8, subband=True, subbands=16, dms_per_subband_dm=16,
                           seed=2),
        serving.BeamConfig(name="single4", channels=192, bandwidth=0.75, samples=2048, dms=96,
                           dm_step=0.3, bits=4, seed=3),
    ]


def test_stream_bytes_and_admission_refusal(engine):
    cfg = small_beams()[0]
    nbytes, tail = serving.stream_bytes(cfg)
    obs, shifts, _, zapped = cfg.tables()
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, cfg.padding, shifts)
    assert tail >= lay.max_delay and tail <= cfg.samples
    ring = cfg.channels * dd.pad(cfg.samples + tail, cfg.padding)
    out = cfg.dms * dd.pad(cfg.samples, cfg.padding // 4) * 4
    assert nbytes == ring + out
    sub = small_beams()[1]
    nb2, _ = serving.stream_bytes(sub)
    assert nb2 > 0
    server = serving.Server(budget_bytes=nbytes - 1)
    with pytest.raises(dd.DedispersionError) as e:
        server.admit(cfg)
    assert e.value.status == _abi.DD_ERR_OVER_BUDGET
    assert server.used == 0 and not server.streams


def batch_data(cfg, k):
    rng = np.random.default_rng(1000 * cfg.seed + k)
    vals = rng.integers(0, 1 << cfg.bits, size=(cfg.channels, cfg.samples), dtype=np.uint16)
    if cfg.bits == 8:
        return vals.astype(np.uint8)
    return syn.pack_subbyte(vals.astype(np.uint8), cfg.bits, cfg.samples * cfg.bits // 8)


def plain_reference(stream, window, oracle):
    """The oracle (the CPU restatement of the reference's loops) on one
    [tail | batch] window: single step, or step one then step two."""
    cfg = stream.cfg
    obs = stream.obs.copy()
    S = cfg.samples
    if not cfg.subband:
        obs.setNrSamplesPerDispersedBatch(S + stream.tail)
        lay = dd.layout(obs, dd.DD_SINGLE_STEP, cfg.bits, cfg.padding)
        inp = np.zeros((cfg.channels, lay.input_row_bytes), np.uint8)
        inp[:, :window.shape[1]] = window
        out = np.zeros(lay.output_bytes // 4, np.float32)
        mapping = np.zeros(lay.mapping_row_elems, np.uint32)
        oracle.dedispersion(obs.c, stream.zapped, mapping, inp.reshape(-1), out, stream.shifts,
                            cfg.padding, cfg.bits)
        return out.reshape(-1, lay.output_row_elems)[:, :S]
    s1 = S + serving_tail_step_two(stream)
    obs.setNrSamplesPerBatch(s1, True)
    obs.setNrSamplesPerDispersedBatch(S + stream.tail, True)
    lay1 = dd.layout(obs, dd.DD_STEP_ONE, cfg.bits, cfg.padding)
    inp = np.zeros((cfg.channels, lay1.input_row_bytes), np.uint8)
    inp[:, :window.shape[1]] = window
    mid = np.zeros(lay1.output_bytes // 4, np.float32)
    oracle.step_one(obs.c, stream.zapped, inp.reshape(-1), mid, stream.shifts, cfg.padding,
                    cfg.bits)
    lay2 = dd.layout(obs, dd.DD_STEP_TWO, 32, cfg.padding)
    out = np.zeros(lay2.output_bytes // 4, np.float32)
    mapping = np.zeros(lay2.mapping_row_elems, np.uint32)
    oracle.step_two(obs.c, mapping, mid, out, stream.shifts2, cfg.padding)
    return out.reshape(-1, lay2.output_row_elems)[:, :S]


def serving_tail_step_two(stream):
    """Step-two max delay (S1 - S) of a subband stream."""
    lay = dd.layout(stream.obs, dd.DD_STEP_TWO, 32, stream.cfg.padding, stream.shifts2)
    return lay.max_delay


@pytest.mark.gpu
@pytest.mark.parametrize("double_buffer", [False, True])
def test_served_batches_equal_oracle(gpu, oracle, double_buffer):
    pytest.importorskip("torch")
    server = serving.Server(budget_bytes=150 * 10**9)
    beams = [dataclasses.replace(c, double_buffer=double_buffer) for c in small_beams()]
    for cfg in beams:
        server.admit(cfg)
    nb = 4
    inputs = {}
    outputs = {}

    def source(b, k, staging):
        data = batch_data(beams[b], k)
        staging[:, :data.shape[1]] = data
        inputs[(b, k)] = data

    def consumer(b, k, out):
        outputs[(b, k)] = out.copy()

    schedule = serving.poisson_schedule(len(beams), nb, period=0.05, jitter=0.01, seed=5)
    report = server.serve(schedule, source, consumer, time_compression=1.0, deadline=2.048)
    s = report.summary()
    assert s["batches"] == len(beams) * nb
    assert s["p99_latency_s"] < 2.048
    for b, stream in enumerate(server.streams):
        cfg = stream.cfg
        per = 8 // cfg.bits if cfg.bits < 8 else 1
        tail_b = stream.tail // per
        prev = np.zeros((cfg.channels, tail_b), np.uint8)
        for k in range(nb):
            cur = inputs[(b, k)]
            window = np.concatenate([prev, cur], axis=1)
            want = plain_reference(stream, window, oracle)
            got = outputs[(b, k)]
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (cfg.name, k)
            prev = window[:, window.shape[1] - tail_b:] if tail_b else prev
    server.close()


@pytest.mark.gpu
def test_time_major_input_equals_channel_rows(gpu):
    """A stream fed file-order blocks (time-major, channels descending) gives
    the same outputs as one fed channel rows, single step and subband."""
    torch = pytest.importorskip("torch")
    cs = torch.cuda.Stream()
    for cfg in [c for c in small_beams() if c.bits == 8][:2]:
        a, b = serving.Stream(cfg), serving.Stream(cfg)
        nb = b.device_bytes
        b.set_time_major(reverse=True)
        assert b.device_bytes == nb + cfg.samples * cfg.channels
        assert b.staging.shape == (cfg.samples, cfg.channels)
        for k in range(3):
            data = batch_data(cfg, k)
            a.staging[:, :cfg.samples] = data
            b.staging[:] = data[::-1].T
            a.push(cs)
            b.push(cs)
            cs.synchronize()
            assert np.array_equal(a.output.view(np.uint32), b.output.view(np.uint32)), (cfg.name, k)
        a.close()
        b.close()


@pytest.mark.gpu
def test_double_buffered_stream_equals_single(gpu):
    """Two pushes in flight on one CUDA stream, staged into alternating
    pinned buffers: the same outputs as one buffer pushed batch by batch."""
    torch = pytest.importorskip("torch")
    cs = torch.cuda.Stream()
    for cfg in small_beams()[:2]:
        a, b = serving.Stream(cfg), serving.Stream(cfg)
        b.set_double_buffer(True)
        assert b.nbuf == 2 and b.next_buffer == 0
        outs = []
        for k in range(4):
            data = batch_data(cfg, k)
            a.staging[:, :cfg.samples] = data
            a.push(cs)
            cs.synchronize()
            want = a.output.copy()
            # b: stage batch k while batch k - 1 may still be in flight
            b.staging[:, :cfg.samples] = data
            idx = b.push(cs)
            assert idx == k % 2
            outs.append((idx, want))
            if k % 2 == 1:
                cs.synchronize()
                for i, w in outs:
                    assert np.array_equal(b.outputs[i].view(np.uint32), w.view(np.uint32)), cfg.name
                outs = []
        a.close()
        b.close()


@pytest.mark.gpu
def test_time_major_double_buffered_stream(gpu):
    """File-order blocks into alternating staging buffers, two pushes in
    flight: the same outputs as channel rows pushed one at a time."""
    torch = pytest.importorskip("torch")
    cs = torch.cuda.Stream()
    cfg = small_beams()[1]  # 8-bit subband
    a, b = serving.Stream(cfg), serving.Stream(cfg)
    b.set_time_major(reverse=True)
    b.set_double_buffer(True)
    assert b.staging.shape == (cfg.samples, cfg.channels)
    want, got_idx = [], []
    for k in range(4):
        data = batch_data(cfg, k)
        a.staging[:, :cfg.samples] = data
        a.push(cs)
        cs.synchronize()
        want.append(a.output.copy())
        b.staging[:] = data[::-1].T
        got_idx.append(b.push(cs))
        if k % 2 == 1:
            cs.synchronize()
            for i, w in zip(got_idx, want):
                assert np.array_equal(b.outputs[i].view(np.uint32), w.view(np.uint32))
            want, got_idx = [], []
    a.close()
    b.close()


@pytest.mark.gpu
def test_late_and_dropped_batches(gpu, oracle):
    """Faults injected on the host: beam 0's batch 1 arrives 0.12 s late (its
    deadline is 0.05 s after its nominal arrival), beam 1's batch 2 never
    arrives.  The late batch and the batch queued behind it miss their
    deadlines, the next one does not; the dropped batch is pushed as zeros,
    neither delivered nor timed, and every delivered batch still equals the
    plain path on its window (the ring stays aligned in time)."""
    pytest.importorskip("torch")
    period = 0.05
    beams = small_beams()[:2]
    server = serving.Server(budget_bytes=150 * 10**9)
    for cfg in beams:
        server.admit(cfg)
    nb = 4
    schedule = [(k * period + 0.001 * b, b, k) for k in range(nb) for b in range(len(beams))]
    schedule = serving.inject(schedule, late={(0, 1): 0.12}, dropped=[(1, 2)])
    inputs, outputs = {}, {}

    def source(b, k, staging):
        data = batch_data(beams[b], k)
        staging[:, :data.shape[1]] = data
        inputs[(b, k)] = data

    def consumer(b, k, out):
        outputs[(b, k)] = out.copy()

    report = server.serve(schedule, source, consumer, deadline=period)
    s = report.summary()
    assert s["batches"] == len(beams) * nb - 1 and s["dropped_batches"] == 1
    assert report.dropped == [(1, 2)] and report.late == [(0, 1)]
    assert set(report.misses) == {(0, 1), (0, 2)}, report.misses
    assert (1, 2) not in outputs and (1, 2) not in inputs
    for b, stream in enumerate(server.streams):
        cfg = stream.cfg
        prev = np.zeros((cfg.channels, stream.tail), np.uint8)
        for k in range(nb):
            cur = inputs.get((b, k), np.zeros((cfg.channels, cfg.samples), np.uint8))
            window = np.concatenate([prev, cur], axis=1)
            if (b, k) in outputs:
                want = plain_reference(stream, window, oracle)
                assert np.array_equal(outputs[(b, k)].view(np.uint32),
                                      want.view(np.uint32)), (cfg.name, k)
            prev = window[:, window.shape[1] - stream.tail:] if stream.tail else prev
    server.close()


@pytest.mark.gpu
def test_file_source_serves_files(gpu, oracle, tmp_path):
    """Beams served straight from files (serving.FileSource): a SIGPROC
    filterbank with descending frequencies and a PSRDADA file with ascending
    ones, three batches each plus a partial fourth, read into the streams'
    pinned staging and transposed on the device; every batch equals the
    plain path on its window of the channel rows the files were written
    from (past the end of a file, zeros)."""
    pytest.importorskip("torch")
    from dedispersion_gb300 import ingest
    C, S, nb = 192, 2048, 4
    rng = np.random.default_rng(17)
    rows = [rng.integers(0, 256, size=(C, 3 * S + S // 2), dtype=np.uint8) for _ in range(2)]
    fil, dada = tmp_path / "beam0.fil", tmp_path / "beam1.dada"
    ingest.write_filterbank(str(fil), rows[0][::-1].T, fch1=1300.0 + (C - 1) * 0.5, foff=-0.5,
                            tsamp=81.92e-6)
    ingest.write_dada(str(dada), rows[1].T, freq=1300.0 - 0.25 + C * 0.5 / 2, bw=C * 0.5,
                      tsamp_us=81.92)
    files = [ingest.Filterbank(str(fil)), ingest.Dada(str(dada))]
    assert files[0].reversed and not files[1].reversed
    cfgs = [serving.FileSource.config(f, f"file{i}", samples=S, dms=64, dm_step=0.2, seed=i,
                                      double_buffer=True)
            for i, f in enumerate(files)]
    server = serving.Server(budget_bytes=150 * 10**9)
    for c in cfgs:
        server.admit(c)
    outputs = {}

    def consumer(b, k, out):
        outputs[(b, k)] = out.copy()

    sched = [(0.0, b, k) for k in range(nb) for b in range(2)]
    report = server.serve(sched, serving.FileSource(files), consumer)
    assert report.summary()["batches"] == 2 * nb
    for b, stream in enumerate(server.streams):
        padded = np.zeros((C, nb * S), np.uint8)
        padded[:, :rows[b].shape[1]] = rows[b]
        prev = np.zeros((C, stream.tail), np.uint8)
        for k in range(nb):
            window = np.concatenate([prev, padded[:, k * S:(k + 1) * S]], axis=1)
            want = plain_reference(stream, window, oracle)
            assert np.array_equal(outputs[(b, k)].view(np.uint32), want.view(np.uint32)), (b, k)
            prev = window[:, window.shape[1] - stream.tail:]
    server.close()
