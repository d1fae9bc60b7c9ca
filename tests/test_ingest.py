"""SIGPROC filterbank and PSRDADA ingest: header, observation mapping, reads,
device transpose.

A file written by ``write_filterbank`` (descending frequencies, as most
telescopes write them) must come back unchanged; its channels map onto the
engine's ascending convention (channel c at min_freq + c * bandwidth) by
reversal; and dedispersing the transposed samples equals the oracle on the
same samples rearranged by numpy.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import ingest
from dedispersion_gb300 import synthetic as syn


def _file(tmp_path, samples=700, nchans=96, seed=1, foff=-0.5):
    rng = np.random.default_rng(seed)
    data = rng.integers(0, 256, size=(samples, nchans), dtype=np.uint8)
    path = tmp_path / "beam.fil"
    ingest.write_filterbank(path, data, fch1=1500.0, foff=foff, tsamp=6.4e-5,
                            source_name="B0000+00")
    return path, data


def test_header_and_reads(tmp_path):
    path, data = _file(tmp_path)
    fb = ingest.Filterbank(path)
    assert fb.info.nchans == 96 and fb.info.nbits == 8 and fb.info.nifs == 1
    assert fb.info.nsamples == 700 and fb.info.tsamp == 6.4e-5
    assert fb.info.fch1 == 1500.0 and fb.info.foff == -0.5
    assert fb.info.source_name == b"B0000+00" and fb.reversed
    np.testing.assert_array_equal(fb.read(0, 700), data)
    np.testing.assert_array_equal(fb.read(123, 45), data[123:168])
    with pytest.raises(dd.DedispersionError, match="past the file"):
        fb.read(690, 20)


def test_observation_from_header(tmp_path):
    path, _ = _file(tmp_path)
    obs = ingest.Filterbank(path).observation(dd.Observation())
    assert obs.getNrChannels() == 96
    assert obs.getMinFreq() == pytest.approx(1500.0 - 95 * 0.5)
    assert obs.getChannelBandwidth() == pytest.approx(0.5)
    assert obs.getSamplingTime() == pytest.approx(6.4e-5)
    # ascending files keep their order
    p2, _ = _file(tmp_path, foff=0.25)
    fb2 = ingest.Filterbank(p2)
    assert not fb2.reversed and fb2.observation(dd.Observation()).getMinFreq() == 1500.0


def test_bad_files(tmp_path):
    bad = tmp_path / "bad.fil"
    bad.write_bytes(b"\x05\x00\x00\x00hello")
    with pytest.raises(dd.DedispersionError, match="HEADER_START"):
        ingest.Filterbank(bad)
    path, _ = _file(tmp_path)
    raw = path.read_bytes()
    cut = tmp_path / "cut.fil"
    cut.write_bytes(raw[:40])
    with pytest.raises(dd.DedispersionError, match="truncated"):
        ingest.Filterbank(cut)


def test_two_ifs_reads_the_first(tmp_path):
    def s(x):
        b = x.encode()
        return np.int32(len(b)).tobytes() + b
    data = np.arange(2 * 10 * 8, dtype=np.uint8).reshape(10, 2, 8)  # [t][if][chan]
    hdr = (s("HEADER_START") + s("nchans") + np.int32(8).tobytes() + s("nbits")
           + np.int32(8).tobytes() + s("nifs") + np.int32(2).tobytes() + s("fch1")
           + np.float64(1400).tobytes() + s("foff") + np.float64(-1).tobytes()
           + s("tsamp") + np.float64(1e-4).tobytes() + s("HEADER_END"))
    p = tmp_path / "two.fil"
    p.write_bytes(hdr + data.tobytes())
    fb = ingest.Filterbank(p)
    assert fb.info.nsamples == 10
    np.testing.assert_array_equal(fb.read(2, 5), data[2:7, 0])


def _dada(tmp_path, samples=500, nchan=64, seed=2, bw=-64.0, **kw):
    rng = np.random.default_rng(seed)
    data = rng.integers(0, 256, size=(samples, nchan), dtype=np.uint8)
    path = tmp_path / "beam.dada"
    ingest.write_dada(path, data, freq=1400.0, bw=bw, tsamp_us=64.0, **kw)
    return path, data


def test_dada_header_reads_and_observation(tmp_path):
    path, data = _dada(tmp_path)
    f = ingest.Dada(path)
    assert f.info.nchan == 64 and f.info.nbit == 8 and f.info.nsamples == 500
    assert f.info.header_bytes == 4096 and f.info.tsamp == pytest.approx(64e-6)
    assert f.info.freq == 1400.0 and f.info.bw == -64.0 and f.reversed
    assert f.info.source == b"synthetic"
    np.testing.assert_array_equal(f.read(0, 500), data)
    np.testing.assert_array_equal(f.read(77, 13), data[77:90])
    obs = f.observation(dd.Observation())
    # 64 channels of 1 MHz centred at 1400 MHz: the lowest centre is 1368.5
    assert obs.getNrChannels() == 64 and obs.getMinFreq() == pytest.approx(1368.5)
    assert obs.getChannelBandwidth() == pytest.approx(1.0)
    with pytest.raises(dd.DedispersionError, match="past the file"):
        f.read(490, 20)
    # a larger header, ascending band
    p2, d2 = _dada(tmp_path, bw=32.0, hdr_size=8192, samples=10, nchan=16)
    g = ingest.Dada(p2)
    assert g.info.header_bytes == 8192 and not g.reversed
    np.testing.assert_array_equal(g.read(0, 10), d2)


def test_dada_rejects_what_it_cannot_read(tmp_path):
    bad = tmp_path / "bad.dada"
    bad.write_bytes(b"NCHAN 4\nNBIT 8\n" + b"\0" * 100)
    with pytest.raises(dd.DedispersionError, match="HDR_SIZE"):
        ingest.Dada(bad)
    p, _ = _dada(tmp_path, extra={"NPOL": "2"})
    with pytest.raises(dd.DedispersionError, match="NPOL 2"):
        ingest.Dada(p)
    p, _ = _dada(tmp_path, extra={"ORDER": "FPT"})
    with pytest.raises(dd.DedispersionError, match="ORDER FPT"):
        ingest.Dada(p)


@pytest.mark.gpu
@pytest.mark.parametrize("nchans,samples,row_bytes,offset", [
    (200, 1000, 1280, 100),   # 4-byte aligned: the word kernel
    (200, 1003, 1280, 100),   # word kernel, ragged last sample word
    (198, 1000, 1283, 101),   # unaligned: the byte kernel
])
def test_device_transpose(gpu, tmp_path, nchans, samples, row_bytes, offset):
    torch = pytest.importorskip("torch")
    path, data = _file(tmp_path, samples=samples, nchans=nchans, seed=4)
    fb = ingest.Filterbank(path)
    d_rows = torch.zeros(nchans * row_bytes, dtype=torch.uint8, device="cuda")
    fb.to_rows(torch.from_numpy(fb.read(0, samples).copy()).cuda(), d_rows, row_bytes, offset)
    torch.cuda.synchronize()
    rows = d_rows.cpu().numpy().reshape(nchans, row_bytes)
    np.testing.assert_array_equal(rows[:, offset:offset + samples], data.T[::-1])
    assert not rows[:, :offset].any() and not rows[:, offset + samples:].any()


@pytest.mark.gpu
def test_filterbank_to_dedispersion_matches_oracle(gpu, oracle, tmp_path):
    """A dispersed pulse written in file order (descending frequency) and
    dedispersed from the device transpose: bit-exact to the oracle on the
    numpy-arranged rows, and the pulse is the brightest DM."""
    torch = pytest.importorskip("torch")
    obs = syn.make_observation(256, 1300.0, 0.5, 6.4e-5, 2048, 128, 0.0, 0.5, padding=128)
    shifts = dd.getShifts(obs, 128)
    rows = syn.make_input(obs, 8, 128, seed=5, mean=100.0, sigma=15.0, pulses=1, shifts=shifts)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, 128, shifts)
    S_disp = obs.getNrSamplesPerDispersedBatch()
    chan_major = rows.reshape(256, lay.input_row_bytes)[:, :S_disp]
    fmax = 1300.0 + 255 * 0.5
    path = tmp_path / "pulse.fil"
    ingest.write_filterbank(path, chan_major[::-1].T, fch1=fmax, foff=-0.5, tsamp=6.4e-5)
    fb = ingest.Filterbank(path)
    obs2 = fb.observation(obs.copy())
    assert obs2.getMinFreq() == pytest.approx(1300.0)
    d_in = torch.zeros(lay.input_bytes, dtype=torch.uint8, device="cuda")
    fb.to_rows(torch.from_numpy(fb.read(0, S_disp).copy()).cuda(), d_in,
               lay.input_row_bytes, 0)
    zapped = np.zeros(lay.zapped_elems, np.uint32)
    mapping = syn.identity_mapping(obs, 128)
    p = dd.Plan(obs, dd.DD_SINGLE_STEP, 8, 128)
    p.setShifts(shifts)
    p.setZappedChannels(zapped)
    p.setBeamMapping(mapping)
    d_out = torch.zeros(lay.output_bytes // 4, dtype=torch.float32, device="cuda")
    p.run(d_in, d_out)
    p.check()
    want = np.zeros(lay.output_bytes // 4, np.float32)
    oracle.dedispersion(obs.c, zapped, mapping, rows, want, shifts, 128, 8)
    got = d_out.cpu().numpy()
    row = lay.output_row_elems
    np.testing.assert_array_equal(got.reshape(-1, row)[:, :2048].view(np.uint32),
                                  want.reshape(-1, row)[:, :2048].view(np.uint32))
    p.close()


@pytest.mark.gpu
def test_dada_to_dedispersion_matches_oracle(gpu, oracle, tmp_path):
    """The same dispersed pulse through a PSRDADA file (descending band)."""
    torch = pytest.importorskip("torch")
    obs = syn.make_observation(256, 1300.0, 0.5, 6.4e-5, 2048, 128, 0.0, 0.5, padding=128)
    shifts = dd.getShifts(obs, 128)
    rows = syn.make_input(obs, 8, 128, seed=6, mean=100.0, sigma=15.0, pulses=1, shifts=shifts)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, 128, shifts)
    S_disp = obs.getNrSamplesPerDispersedBatch()
    chan_major = rows.reshape(256, lay.input_row_bytes)[:, :S_disp]
    # channel centres 1300 + c * 0.5 MHz: a band of 128 MHz centred at 1363.75
    path = tmp_path / "pulse.dada"
    ingest.write_dada(path, chan_major[::-1].T, freq=1363.75, bw=-128.0, tsamp_us=64.0)
    f = ingest.Dada(path)
    assert f.observation(obs.copy()).getMinFreq() == pytest.approx(1300.0)
    d_in = torch.zeros(lay.input_bytes, dtype=torch.uint8, device="cuda")
    f.to_rows(torch.from_numpy(f.read(0, S_disp).copy()).cuda(), d_in, lay.input_row_bytes, 0)
    zapped = np.zeros(lay.zapped_elems, np.uint32)
    mapping = syn.identity_mapping(obs, 128)
    p = dd.Plan(obs, dd.DD_SINGLE_STEP, 8, 128)
    p.setShifts(shifts)
    p.setZappedChannels(zapped)
    p.setBeamMapping(mapping)
    d_out = torch.zeros(lay.output_bytes // 4, dtype=torch.float32, device="cuda")
    p.run(d_in, d_out)
    p.check()
    want = np.zeros(lay.output_bytes // 4, np.float32)
    oracle.dedispersion(obs.c, zapped, mapping, rows, want, shifts, 128, 8)
    row = lay.output_row_elems
    np.testing.assert_array_equal(d_out.cpu().numpy().reshape(-1, row)[:, :2048],
                                  want.reshape(-1, row)[:, :2048])
    p.close()
