"""Host-buffer calls split into chunks of time tiles (run_sync): each
chunk's input samples are copied in just before it (the first chunk needs
its tiles plus the largest delay), and its output columns go back to the host
while later chunks compute.

The result must equal the oracle (include/Dedispersion.hpp:70-176) and the
device plan path bit for bit in single step (3 synthesized beams, a partial
last DM tile and a partial last time tile), step one and step two; a small
problem keeps one launch and one copy each way.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from helpers import engine_run, oracle_run, single_case, step_one_case, step_two_case

pytestmark = pytest.mark.gpu


def _plan_out(case):
    torch = pytest.importorskip("torch")
    p = dd.Plan(case.obs, case.mode, case.bits, case.padding)
    p.setShifts(case.shifts)
    if case.mode != dd.DD_STEP_TWO:
        p.setZappedChannels(case.zapped)
    if case.mode != dd.DD_STEP_ONE:
        p.setBeamMapping(case.mapping)
    d_in = torch.from_numpy(np.ascontiguousarray(case.inp).view(np.uint8).reshape(-1)).cuda()
    d_out = torch.zeros(case.out_elems, dtype=torch.float32, device="cuda")
    p.run(d_in, d_out)
    p.check()
    p.close()
    return d_out.cpu().numpy()


def test_single_step_chunks_across_beams_and_partial_tiles(gpu, oracle):
    # 3 synthesized beams x 1000 DMs (a partial last DM tile) x 16300 samples
    # (a partial last time tile): 64 time tiles in 16 chunks, 3072 tiles.
    case = single_case(C=256, D=1000, S=16300, bits=8, padding=128, beams=2, sbeams=3, zap=0.05,
                       seed=17, dist="uniform")
    got = engine_run(case)
    for want in (_plan_out(case), oracle_run(oracle, case)):
        np.testing.assert_array_equal(case.valid(got).view(np.uint32),
                                      case.valid(want).view(np.uint32))


def test_step_one_chunks(gpu, oracle):
    case = step_one_case(bits=8, padding=128, seed=5, C=1024, SB=32, D1=64, step1=3.2, D2=16,
                         step2=0.2, S=32000, beams=2, sdisp_multiple=16)
    got = engine_run(case)
    for want in (_plan_out(case), oracle_run(oracle, case)):
        np.testing.assert_array_equal(case.valid(got).view(np.uint32),
                                      case.valid(want).view(np.uint32))


def test_step_two_chunks(gpu, oracle):
    case = step_two_case(padding=128, seed=9, float_values=True, C=1024, SB=32, D1=8, D2=256,
                         S=16384, beams=2, sbeams=2)
    got = engine_run(case)
    for want in (_plan_out(case), oracle_run(oracle, case)):
        np.testing.assert_array_equal(case.valid(got).view(np.uint32),
                                      case.valid(want).view(np.uint32))


def test_small_problem_single_launch(gpu, oracle):
    case = single_case(C=64, D=40, S=512, bits=4, padding=64, sbeams=2, beams=2, seed=3)
    got = engine_run(case)
    for want in (_plan_out(case), oracle_run(oracle, case)):
        np.testing.assert_array_equal(case.valid(got).view(np.uint32),
                                      case.valid(want).view(np.uint32))


def _pinned_like(out):
    torch = pytest.importorskip("torch")
    t = torch.full((out.size,), -3.0, dtype=torch.float32).pin_memory()
    return t, t.numpy()


@pytest.mark.parametrize("kind", ["single_chunked", "single_small", "step_one_chunked"])
def test_pinned_output_written_by_the_kernels(gpu, oracle, kind):
    """With a pinned host output on a device that reaches host memory through
    the host's page tables, the kernels write the output straight into it
    (no device buffer, no copy back); the result is the oracle's bit for bit
    and the row padding is left as it was."""
    if kind == "single_chunked":
        case = single_case(C=256, D=1000, S=16300, bits=8, padding=128, beams=2, sbeams=3,
                           zap=0.05, seed=19)
    elif kind == "single_small":
        case = single_case(C=64, D=40, S=500, bits=4, padding=64, sbeams=2, beams=2, seed=23)
    else:
        case = step_one_case(bits=8, padding=128, seed=29, C=1024, SB=32, D1=64, step1=3.2,
                             D2=16, step2=0.2, S=32000, beams=2, sdisp_multiple=16)
    keep, out = _pinned_like(case.output())
    if case.mode == dd.DD_SINGLE_STEP:
        dd.dedispersion(case.obs, case.zapped, case.mapping, case.inp, out, case.shifts,
                        case.padding, case.bits)
    else:
        dd.subbandDedispersionStepOne(case.obs, case.zapped, case.inp, out, case.shifts,
                                      case.padding, case.bits)
    want = oracle_run(oracle, case)
    np.testing.assert_array_equal(case.valid(out).view(np.uint32),
                                  case.valid(want).view(np.uint32))
    pad = out.reshape(case.out_rows, case.out_row)[:, case.nr_samples:]
    assert (pad == -3.0).all()
    del keep
