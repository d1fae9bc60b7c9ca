"""Host check of the shared-partial-sum stage tables (no GPU).

tests/cpp/shared_tables_test.cu replays the kernel's indexing over the tables
the library builds (dd_shared_plan.cu) and compares every output sample of
the covered tiles with the direct sum.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import build as ddbuild
from dedispersion_gb300 import synthetic as syn
from helpers import single_case

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = ddbuild.nvcc()
    if not shutil.which(nvcc) and not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("stt") / "shared_tables_test"
    cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-o", str(exe),
           str(ROOT / "tests/cpp/shared_tables_test.cu"),
           str(ROOT / "dedispersion_gb300/csrc/dd_shared_plan.cu")]
    subprocess.run(cmd, check=True, capture_output=True, timeout=600)
    return exe


def run(exe, tmp_path, shifts, dms, samples, first, step, cfg, seed=5, time_tiles=1):
    f = tmp_path / "shifts.f32"
    np.asarray(shifts, np.float32).tofile(f)
    p = subprocess.run([str(exe), str(f), str(len(shifts)), str(dms), str(samples), str(first),
                        str(step), *map(str, cfg), str(seed), str(time_tiles)],
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0 and p.stdout.startswith("PASS"), p.stdout + p.stderr
    return dict(kv.split("=") for kv in p.stdout.split()[1:])


@pytest.mark.parametrize("cfg", [(4, 4, 16), (8, 2, 16)])
def test_full_size_table(harness, tmp_path, cfg):
    """1536 channels (5 % zapped) x 2048 DMs at 0.2: every DM tile, one time tile."""
    obs = syn.large_observation(128)
    sh = dd.getShifts(obs, 128)[:1536]
    z = syn.zapped_mask(1536, 0.05, 7, 128)[:1536]
    info = run(harness, tmp_path, sh[z == 0], 2048, 24576, 0.0, 0.2, cfg)
    # fewer than half the direct form's adds (1459 per DM-sample)
    per_ds = (int(info["adds_partial"]) + int(info["adds_series"])) / (2048 * 64 * cfg[0])
    assert per_ds < 1459 / 2


def test_short_subgroups_large_relative_delays(harness, tmp_path):
    """4 MHz channels at 400 MHz: relative delays within eight channels pass
    the limit at high DMs, so subgroups shrink; two time tiles."""
    case = single_case(C=64, D=256, S=512, bits=8, padding=128, zap=0.0, seed=6, step=0.012,
                       fmin=400.0, bw=4.0)
    for cfg in [(4, 4, 16), (8, 2, 16)]:
        run(harness, tmp_path, case.shifts[:64], 256, 512, 0.0, 0.012, cfg, time_tiles=2)


def test_nonzero_first_dm(harness, tmp_path):
    obs = syn.large_observation(128)
    sh = dd.getShifts(obs, 128)[:1536:3]
    run(harness, tmp_path, sh, 300, 1000, 37.5, 0.35, (2, 4, 16), time_tiles=4)


def test_small_shared_memory_budget(harness, tmp_path):
    """A budget that holds few series: subgroups shrink so that one fits."""
    obs = syn.large_observation(128)
    sh = dd.getShifts(obs, 128)[:1536:2]
    f = tmp_path / "shifts.f32"
    np.asarray(sh, np.float32).tofile(f)
    p = subprocess.run([str(harness), str(f), str(len(sh)), "512", "2048", "0", "0.2", "4", "4",
                        "16", "3", "2", "160000"], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0 and p.stdout.startswith("PASS"), p.stdout + p.stderr
