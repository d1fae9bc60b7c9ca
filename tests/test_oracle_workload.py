"""The oracle stands alone: its struct mirrors match the engine's ABI structs,
and its numpy-only workload builder (used by the CPU baseline and the
reference arm of bench.py, which must not load the engine) draws the same
bytes as the engine's seeded generator."""
import ctypes as C
import subprocess
import sys

import numpy as np

import dedispersion_gb300 as dd
from dedispersion_gb300 import _abi
from dedispersion_gb300 import synthetic as syn
from oracle import types as otypes
from oracle import workload as owl


def _layout(struct):
    return [(name, getattr(struct, name).offset, getattr(struct, name).size)
            for name, _ in struct._fields_]


def test_struct_mirrors_match_the_abi():
    assert _layout(otypes.DdObservation) == _layout(_abi.DdObservation)
    assert C.sizeof(otypes.DdObservation) == C.sizeof(_abi.DdObservation)
    assert _layout(otypes.DdConf) == _layout(_abi.DdConf)


def test_oracle_import_does_not_load_the_engine():
    code = ("import sys, oracle, oracle.workload; "
            "print(any(m == 'dedispersion_gb300' or m.startswith('dedispersion_gb300.') "
            "for m in sys.modules))")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         check=True, cwd=str(__import__("pathlib").Path(__file__).parents[1]))
    assert out.stdout.strip() == "False"


def test_workload_equals_engine_generator(oracle):
    padding = 128
    o, sh, z, m, inp = owl.single_step(seed=1, padding=padding)
    obs = syn.large_observation(padding)
    shifts = dd.getShifts(obs, padding)
    assert np.array_equal(sh.view(np.uint32), shifts.view(np.uint32))
    assert bytes(o) == bytes(obs.c)
    assert np.array_equal(z, syn.zapped_mask(1536, 0.05, 7, padding))
    assert np.array_equal(m, syn.identity_mapping(obs, padding))
    want = syn.make_input(obs, 8, padding, seed=1, mean=128.0, sigma=20.0, pulses=20,
                          shifts=shifts)
    assert inp.dtype == want.dtype and np.array_equal(inp, want)
