"""Golden vectors made by the reference's own CPU code (tests/golden/make_golden.py).

The reference tree has no stored golden vectors (its only test compares the
OpenCL kernel with its CPU templates at run time), so the fixtures were
generated by running those templates, compiled unmodified, on seeded inputs.
The CPU tests pin the oracle restatement to them on any machine; the GPU
tests pin the engine.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import synthetic as syn

from helpers import engine_run, oracle_run, single_case, step_one_case, step_two_case

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"


@pytest.fixture(scope="module")
def golden():
    g = np.load(GOLDEN)
    manifest = json.loads(bytes(g["manifest"]).decode())
    return g, manifest


def build(kind, kw):
    kw = dict(kw)
    if kw.get("mapping") == "zeros":
        kw["mapping"] = np.zeros(dd.pad(kw["C"], kw["padding"] // 4), np.uint32)
    return {"single": single_case, "one": step_one_case, "two": step_two_case}[kind](**kw)


def cases(manifest):
    return [k for k in manifest if not k.startswith("_")]


def test_golden_inputs_regenerate(engine, golden):
    g, manifest = golden
    for name in cases(manifest):
        m = manifest[name]
        case = build(m["kind"], m["kwargs"])
        assert hashlib.sha256(case.inp.tobytes()).hexdigest() == m["input_sha256"], name


def test_oracle_matches_golden(engine, oracle, golden):
    g, manifest = golden
    for name in cases(manifest):
        m = manifest[name]
        case = build(m["kind"], m["kwargs"])
        got = oracle_run(oracle, case, threads=2)
        want = g[f"{name}__out"]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name


def test_shift_tables_match_golden(engine, oracle, golden):
    g, manifest = golden
    obs1, obs2 = syn.small_observation(128), syn.large_observation(128)
    obs2s = syn.large_observation(128, subbands=True)
    pairs = [(dd.getShifts(obs1, 128), "shifts_small_pad128"),
             (dd.getShifts(obs2, 128), "shifts_large_pad128"),
             (dd.getShifts(obs2s, 128), "shifts_large_subband_pad128"),
             (dd.getShiftsStepTwo(obs2s, 128), "shifts2_large_subband_pad128")]
    for got, key in pairs:
        np.testing.assert_array_equal(got.view(np.uint32), g[key].view(np.uint32), key)
    np.testing.assert_array_equal(oracle.shifts(obs2.c, 128).view(np.uint32),
                                  g["shifts_large_pad128"].view(np.uint32))
    ds = manifest["_dispersed_samples"]
    assert obs1.getNrSamplesPerDispersedBatch() == ds["small"] == 1130
    assert obs2.getNrSamplesPerDispersedBatch() == ds["large"] == 29530
    assert obs2s.getNrSamplesPerBatch(True) == ds["large_subband_S1"]
    assert obs2s.getNrSamplesPerDispersedBatch(True) == ds["large_subband_S1_disp"]


@pytest.mark.gpu
def test_engine_matches_golden(gpu, golden):
    g, manifest = golden
    for name in cases(manifest):
        m = manifest[name]
        case = build(m["kind"], m["kwargs"])
        got = engine_run(case)
        want = g[f"{name}__out"]
        gv, wv = case.valid(got), case.valid(want)
        assert np.array_equal(gv.view(np.uint32), wv.view(np.uint32)), name
