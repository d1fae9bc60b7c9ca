"""The C++ drop-in surface (include/dedispersion_gb300.hpp) and its
DedispersionTest twin (tests/cpp/dedispersion_test.cpp)."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
SRC = ROOT / "tests" / "cpp" / "dedispersion_test.cpp"


def compile_test(out: Path, syntax_only: bool = False, src: Path = SRC) -> None:
    cmd = ["g++", "-std=c++14", "-O2", "-Wall", "-Wno-unused-result", f"-I{ROOT / 'include'}",
           f"-I{CUDA / 'include'}", str(src)]
    if syntax_only:
        cmd += ["-fsyntax-only"]
    else:
        cmd += ["-o", str(out), f"-L{ROOT / 'dedispersion_gb300'}", "-ldedisp_gb300",
                f"-Wl,-rpath,{ROOT / 'dedispersion_gb300'}", f"-L{ROOT / 'oracle'}", "-lddoracle",
                f"-Wl,-rpath,{ROOT / 'oracle'}", f"-L{CUDA / 'lib64'}", "-lcudart_static",
                "-ldl", "-lrt", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_header_compiles_as_cpp14(engine):
    compile_test(Path("/dev/null"), syntax_only=True)
    compile_test(Path("/dev/null"), syntax_only=True, src=ROOT / "tests" / "cpp" / "subband_test.cpp")


def test_header_declares_the_reference_surface():
    text = (ROOT / "include" / "dedispersion_gb300.hpp").read_text()
    for name in ["class Observation", "class DedispersionConf", "getShifts(", "getShiftsStepTwo(",
                 "void dedispersion(", "void subbandDedispersionStepOne(",
                 "void subbandDedispersionStepTwo(", "readTunedDedispersionConf(",
                 "tunedDedispersionConf", "void subbandDedispersion("]:
        assert name in text, name


COMMON = ["-padding", "128", "-beams", "1", "-sampling_time", "0.00008192", "-min_freq", "1220",
          "-channel_bandwidth", "0.1953125", "-samples", "2048"]

RUNS = [
    ["-single_step", "-random", "-synthesized_beams", "1", "-channels", "256", "-dms", "96",
     "-dm_first", "0", "-dm_step", "0.4"],
    ["-single_step", "-synthesized_beams", "1", "-channels", "256", "-dms", "64",
     "-dm_first", "0", "-dm_step", "0.4", "-threadsD0", "32", "-threadsD1", "8", "-itemsD0", "8",
     "-itemsD1", "4", "-unroll", "16"],
    ["-single_step", "-random", "-input_bits", "4", "-synthesized_beams", "1", "-channels", "128",
     "-dms", "40", "-dm_first", "0", "-dm_step", "0.5"],
    ["-single_step", "-random", "-input_bits", "2", "-synthesized_beams", "1", "-channels", "128",
     "-dms", "40", "-dm_first", "1", "-dm_step", "0.5"],
    ["-step_one", "-random", "-subbands", "8", "-channels", "256", "-subbanding_dms", "16",
     "-subbanding_dm_first", "0", "-subbanding_dm_step", "3.2", "-dms", "16", "-dm_first", "0",
     "-dm_step", "0.2"],
    ["-step_two", "-random", "-synthesized_beams", "1", "-subbands", "8", "-channels", "256",
     "-subbanding_dms", "16", "-dms", "16", "-dm_first", "0", "-dm_step", "0.2"],
]


@pytest.mark.gpu
@pytest.mark.parametrize("run", RUNS, ids=lambda r: "_".join(r[:3]))
def test_dedispersion_test_twin_passes(gpu, oracle, tmp_path, run):
    exe = tmp_path / "dedispersion_test"
    compile_test(exe)
    zfile = tmp_path / "zapped.txt"
    zfile.write_text("3 17\n100 101 255\n")
    args = [str(exe), *COMMON, *run]
    if "-step_two" not in run:
        args += ["-zapped_channels", str(zfile)]
    proc = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert "TEST PASSED." in proc.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("argv", [["256", "8", "16", "16", "8", "1", "1", "3"],
                                  ["512", "4", "7", "12", "8", "2", "3", "5"],
                                  ["256", "8", "9", "16", "4", "2", "2", "7"]],
                         ids=["8bit", "odd_coarse_multibeam", "4bit"])
def test_subband_one_call_matches_oracle(gpu, oracle, tmp_path, argv):
    exe = tmp_path / "subband_test"
    compile_test(exe, src=ROOT / "tests" / "cpp" / "subband_test.cpp")
    proc = subprocess.run([str(exe), *argv], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert "TEST PASSED." in proc.stdout
