"""The C ABI library: loads, exports every declared entry point, and its
host-only calls (geometry, layouts, tuned-conf files, argument checks) work
without a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import _abi
from dedispersion_gb300 import synthetic as syn

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(dd_[a-z_0-9]+)\s*\(", text,
                            flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(engine):
    lib = C.CDLL(str(_abi.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert set(names) <= set(_abi.SIGNATURES), set(names) - set(_abi.SIGNATURES)


def test_version_and_pad(engine):
    assert _abi.lib().dd_version() == 1
    assert dd.pad(29530, 128) == 29568
    assert dd.pad(10, 0) == 10
    assert dd.pad(0, 16) == 0


def test_layouts_follow_reference(engine):
    obs = syn.large_observation(128)
    lay = dd.layout(obs, dd.DD_SINGLE_STEP, 8, 128, dd.getShifts(obs, 128))
    assert lay.input_row_bytes == 29568
    assert lay.input_bytes == 1536 * 29568
    assert lay.output_row_elems == 24576
    assert lay.output_bytes == 2048 * 24576 * 4
    assert lay.max_delay == 4953
    assert lay.required_dispersed_samples <= obs.getNrSamplesPerDispersedBatch()
    lay4 = dd.layout(obs, dd.DD_SINGLE_STEP, 4, 128)
    assert lay4.input_row_bytes == dd.pad((29530 + 1) // 2, 128)
    lay16 = dd.layout(obs, dd.DD_SINGLE_STEP, 16, 128)
    assert lay16.input_row_bytes == dd.pad(29530, 64) * 2


def test_frequency_getters(engine):
    obs = syn.large_observation(0, subbands=True)
    assert obs.getMaxFreq() == np.float32(1220.0) + np.float32(1535) * np.float32(0.1953125)
    assert obs.getSubbandBandwidth() == np.float32(48) * np.float32(0.1953125)
    assert obs.getSubbandMaxFreq() == obs.getMaxFreq()


def test_conf_print_and_tuned_file_roundtrip(engine, tmp_path):
    c = dd.DedispersionConf(unroll=16, nrThreadsD1=8, nrItemsD0=16, nrItemsD1=4)
    assert c.print() == "0 1 16 32 8 1 16 4 1"
    path = tmp_path / "tuned.conf"
    path.write_text("# comment line\n\n")
    dd.writeTunedDedispersionConf(str(path), "GB300", 2048, c)
    dd.writeTunedDedispersionConf(str(path), "GB300", 128, dd.DedispersionConf(unroll=8))
    dd.writeTunedDedispersionConf(str(path), "GB300", 2048, dd.DedispersionConf(unroll=4))
    got = dd.readTunedDedispersionConf(str(path), "GB300", 2048)
    assert got == c  # first line of a (device, nrDMs) pair wins
    assert dd.readTunedDedispersionConf(str(path), "GB300", 128).unroll == 8
    with pytest.raises(dd.DedispersionError) as e:
        dd.readTunedDedispersionConf(str(path), "GB300", 7)
    assert e.value.status == _abi.DD_ERR_NOT_FOUND
    with pytest.raises(dd.DedispersionError) as e:
        dd.readTunedDedispersionConf(str(tmp_path / "missing.conf"), "GB300", 7)
    assert e.value.status == _abi.DD_ERR_FILE


def test_tuned_file_matches_reference_reader(engine, ref, tmp_path):
    path = tmp_path / "tuned.conf"
    path.write_text("GB300 2048 0 1 16 32 8 1 16 4 1\n# x\nGB300 2048 0 0 4 32 4 1 8 2 1\n"
                    "GB300 128 0 1 8 32 8 1 8 2 1\n")
    for nr in (2048, 128):
        conf = _abi.DdConf()
        printed = C.create_string_buffer(256)
        assert ref.ddref_read_tuned_conf(str(path).encode(), b"GB300", nr, C.byref(conf),
                                         printed, 256) == 0
        ours = dd.readTunedDedispersionConf(str(path), "GB300", nr)
        assert ours == dd.DedispersionConf.from_c(conf)
        assert ours.print() == printed.value.decode()


def test_malformed_tuned_line_is_an_error(engine, tmp_path):
    path = tmp_path / "bad.conf"
    path.write_text("GB300 2048 0 1 16\n")
    with pytest.raises(dd.DedispersionError) as e:
        dd.readTunedDedispersionConf(str(path), "GB300", 2048)
    assert e.value.status == _abi.DD_ERR_FILE


def test_argument_errors_without_device(engine):
    obs = syn.small_observation()
    bad = obs.copy()
    bad.setDMRange(8, -1.0, 0.25)
    with pytest.raises(dd.DedispersionError) as e:
        dd.layout(bad, dd.DD_SINGLE_STEP, 8, 0)
    assert e.value.status == _abi.DD_ERR_INVALID_ARGUMENT
    with pytest.raises(dd.DedispersionError) as e:
        dd.layout(obs, dd.DD_SINGLE_STEP, 3, 0)
    assert e.value.status == _abi.DD_ERR_UNSUPPORTED


def test_no_cpu_fallback(engine):
    """On a host without a GPU every compute entry point fails loudly."""
    if dd.device_count() > 0:
        pytest.skip("a GPU is present")
    obs = syn.small_observation()
    inp = syn.make_input(obs, 8, 0, seed=1)
    out = syn.output_buffer(obs, dd.DD_SINGLE_STEP, 0)
    with pytest.raises(dd.DedispersionError) as e:
        dd.dedispersion(obs, np.zeros(256, np.uint32), np.zeros(256, np.uint32), inp, out,
                        dd.getShifts(obs, 0), 0, 8)
    assert e.value.status == _abi.DD_ERR_NO_DEVICE
    with pytest.raises(dd.DedispersionError) as e:
        dd.Plan(obs, dd.DD_SINGLE_STEP, 8, 0)
    assert e.value.status == _abi.DD_ERR_NO_DEVICE


def test_kernel_registry(engine):
    ks = dd.kernels()
    assert any(k.elem_bits == 8 for k in ks)
    assert any(k.elem_bits == 16 for k in ks)
    assert any(k.elem_bits == 32 for k in ks)
    for k in ks:
        assert k.conf.nrThreadsD0 == 32
        assert k.conf.localMem
