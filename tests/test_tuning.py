"""The exhaustive tuner (DedispersionTuning's role) and the learned tuner."""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import tuning

ROOT = Path(__file__).resolve().parents[1]


def test_study_shapes_are_seeded_and_in_range(engine):
    a, b = tuning.study_shapes(50), tuning.study_shapes(50)
    assert a == b
    for s in a:
        assert 256 <= s.channels <= 4096 and s.bits in (2, 4, 8, 32)
        assert 4096 <= s.samples <= 65536 and 32 <= s.dms <= 8192
        assert s.subbands in (0, 16, 32, 64, 128)
        if s.subbands:
            assert s.channels % s.subbands == 0


def test_features_distinguish_configurations(engine):
    s = tuning.study_shapes(1)[0]
    ks = tuning.family_kernels(s.mode(), s.bits)
    F = np.stack([tuning.features(s, k.conf, k.name) for k in ks])
    assert np.isfinite(F).all()
    assert len({tuple(r) for r in F}) == len(ks)
    nf, nv = len(tuning.FAMILIES), len(tuning.VARIANTS)
    for k, f in zip(ks, F):
        assert f[-nf:].sum() == 1, k.name                      # one family
        assert f[-nf - nv:-nf].sum() == (1 if k.name.startswith("swar8") else 0), k.name


def test_reference_switches_filter_the_registry(engine):
    """-max_rows/-max_columns/-vector/-max_sample_items/-max_dm_items/
    -max_unroll/-max_items/-min_threads/-max_threads keep exactly the
    configurations the reference's enumeration limits would admit
    (src/DedispersionTuning.cpp:201-283)."""
    import argparse
    ks = tuning.family_kernels(dd.DD_SINGLE_STEP, 8)
    none = argparse.Namespace()
    assert tuning.registry_filter(ks, dd.DD_SINGLE_STEP, 8, none) == ks
    a = tuning._args(["-single_step", "-max_rows", "8", "-max_columns", "32", "-vector", "64",
                      "-max_sample_items", "8", "-max_dm_items", "4", "-max_unroll", "16",
                      "-max_items", "40", "-min_threads", "32", "-max_threads", "1024"])
    kept = tuning.registry_filter(ks, dd.DD_SINGLE_STEP, 8, a)
    assert kept and len(kept) < len(ks)
    for k in ks:
        c = k.conf
        t0, t1 = c.nrThreadsD0, c.nrThreadsD1
        est = c.nrItemsD1 + c.nrItemsD0 * c.nrItemsD1 + 9
        ok = (32 <= t0 <= 32 and t1 <= 8 and t0 * t1 <= 1024 and (t0 * t1) % 64 == 0 and
              c.nrItemsD0 <= 8 and c.nrItemsD1 <= 4 and c.unroll <= 16 and est <= 40)
        assert (k in kept) == ok, k.name
    # sub-byte input adds 4 to the register estimate
    tight = tuning._args(["-single_step", "-max_items", str(min(
        k.conf.nrItemsD1 + k.conf.nrItemsD0 * k.conf.nrItemsD1 + 9 for k in ks))])
    assert tuning.registry_filter(ks, dd.DD_SINGLE_STEP, 8, tight)
    assert not tuning.registry_filter(ks, dd.DD_SINGLE_STEP, 4, tight)


@pytest.mark.gpu
def test_exhaustive_cli_best_line(gpu, tmp_path):
    tuned = tmp_path / "tuned.conf"
    args = [sys.executable, "-m", "dedispersion_gb300.tuning", "-iterations", "2", "-single_step",
            "-padding", "128", "-beams", "1", "-synthesized_beams", "1", "-samples", "4096",
            "-sampling_time", "0.00008192", "-min_freq", "1220", "-channel_bandwidth", "0.5",
            "-channels", "256", "-dms", "128", "-dm_first", "0", "-dm_step", "0.2", "-best",
            "-tuned_file", str(tuned), "-device_name", "GB300"]
    p = subprocess.run(args, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    fields = p.stdout.split()
    assert fields[0] == "128" and len(fields) == 10
    conf = dd.readTunedDedispersionConf(str(tuned), "GB300", 128)
    assert conf.print() == " ".join(fields[1:])


@pytest.mark.gpu
def test_learned_tuner_beats_random_choice(gpu, tmp_path):
    shapes = tuning.study_shapes(48, seed=99)
    # small problems keep the sweep short
    old = tuning.measured_observation
    tuning.measured_observation = lambda s, p: old(s, p, max_dms=64, max_samples=2048)
    try:
        records = tuning.collect(shapes, iterations=2)
    finally:
        tuning.measured_observation = old
    X, y, owner = tuning.dataset(records)
    train = np.arange(36)
    test = np.arange(36, 48)
    t = tuning.LearnedTuner(seed=3)
    t.fit(X[np.isin(owner, train)], y[np.isin(owner, train)], steps=1500)
    rep = tuning.evaluate(records, t, test, k=4)
    assert rep["top_k_vs_best_mean"] >= rep["random_k_vs_best_mean"]
    assert rep["top_k_vs_best_mean"] > 0.8
    assert rep["tuning_time_ratio"] < 0.5
    # a saved model ranks the same after loading
    path = tmp_path / "model.npz"
    t.save(str(path))
    u = tuning.LearnedTuner.load(str(path))
    np.testing.assert_allclose(u.predict(X[:50]), t.predict(X[:50]), rtol=1e-6, atol=1e-6)
    # the CLI times only the model's top 2 and prints a tuned-conf line
    tuned = tmp_path / "tuned.conf"
    args = [sys.executable, "-m", "dedispersion_gb300.tuning", "-iterations", "2", "-single_step",
            "-padding", "128", "-beams", "1", "-synthesized_beams", "1", "-samples", "4096",
            "-sampling_time", "0.00008192", "-min_freq", "1220", "-channel_bandwidth", "0.5",
            "-channels", "256", "-dms", "128", "-dm_first", "0", "-dm_step", "0.2", "-best",
            "-learned", str(path), "-top_k", "2", "-tuned_file", str(tuned)]
    p = subprocess.run(args, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    fields = p.stdout.split()
    assert fields[0] == "128" and len(fields) == 10
    assert "learned: timed 2 of" in p.stderr, p.stderr
    assert dd.readTunedDedispersionConf(str(tuned), "GB300", 128).print() == " ".join(fields[1:])


def test_observation_shape_maps_problems_to_study_features(engine):
    """A user problem maps onto the features the study trained on: single
    step directly; step one as a subband shape whose DM step is the coarse
    step / 32 and whose DM count is coarse DMs x 32 (the study's geometry)."""
    from dedispersion_gb300 import synthetic as syn
    obs = syn.large_observation(128)
    sh = dd.getShifts(obs, 128)
    s = tuning.observation_shape(obs, dd.DD_SINGLE_STEP, 8, sh)
    assert (s.channels, s.dms, s.samples, s.subbands) == (1536, 2048, 24576, 0)
    assert s.dm_step == pytest.approx(0.2) and s.shift0 == pytest.approx(float(sh[0]))
    sub = syn.large_observation(128, subbands=True)
    s1 = tuning.observation_shape(sub, dd.DD_STEP_ONE, 8, dd.getShifts(sub, 128))
    assert (s1.subbands, s1.dms) == (32, 64 * 32) and s1.dm_step == pytest.approx(6.4 / 32)
    assert s1.mode() == dd.DD_STEP_ONE and s.mode() == dd.DD_SINGLE_STEP
    # the study band's default delay constant is used when shift0 is unset
    f_default = tuning.features(tuning.Shape(1536, 2048, 24576, 8, 0, 0.2), *_first(s))
    f_real = tuning.features(s, *_first(s))
    assert f_default.shape == f_real.shape


def _first(shape):
    k = tuning.family_kernels(shape.mode(), shape.bits)[0]
    return k.conf, k.name


def test_shared_adds_ratio_estimate(engine):
    """The shared tile's estimated adds per direct-sum add: at least the
    series adds (1/8), below the direct sum for the study band, rising with
    the DM step (fewer DMs share a delay vector), and the feature is set for
    the shared configurations only."""
    r = [tuning.shared_adds_ratio(1536, 2048, s, 64) for s in (0.05, 0.2, 0.45)]
    assert all(0.125 < x < 1.0 for x in r)
    assert r[0] < r[1] < r[2]
    # 1536 channels, 2048 DMs at 0.2: the plans' own count is 0.21-0.23
    assert 0.18 < r[1] < 0.30
    s = tuning.Shape(channels=1536, dms=2048, samples=24576, bits=8, subbands=0, dm_step=0.2)
    i = tuning.FEATURE_NAMES.index("log2 shared adds ratio")
    for k in tuning.family_kernels(s.mode(), s.bits):
        f = tuning.features(s, k.conf, k.name)
        if k.name.startswith("shared8"):
            assert f[i] < 0
        else:
            assert f[i] == 0
