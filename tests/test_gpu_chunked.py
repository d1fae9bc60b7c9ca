"""Host-buffer calls split into chunks of DM tiles (run_sync): the output
rows each chunk finishes are copied to the host while later chunks compute.

The result must equal the device plan path bit for bit where chunk
boundaries cross synthesized-beam groups and partial DM tiles, in single
step and in step two (whose rows are contiguous in tile order too); a small
problem (one launch) and step one (rows not contiguous) keep one copy.
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from helpers import engine_run, single_case, step_two_case

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


def test_single_step_chunks_across_beams_and_partial_tiles(gpu):
    # 3 synthesized beams x 1000 DMs (a partial last DM tile) x 16384 samples:
    # 48 (beam, DM tile) pairs over 8 chunks, 3072 tiles.
    case = single_case(C=256, D=1000, S=16384, bits=8, padding=128, beams=2, sbeams=3, zap=0.05,
                       seed=17, dist="uniform")
    got = engine_run(case)
    want = _plan_out(case)
    np.testing.assert_array_equal(case.valid(got).view(np.uint32),
                                  case.valid(want).view(np.uint32))


def test_step_two_chunks(gpu):
    case = step_two_case(padding=128, seed=9, float_values=True, C=1024, SB=32, D1=8, D2=256,
                         S=16384, beams=2, sbeams=2)
    got = engine_run(case)
    want = _plan_out(case)
    np.testing.assert_array_equal(case.valid(got).view(np.uint32),
                                  case.valid(want).view(np.uint32))


def test_small_problem_single_launch(gpu):
    case = single_case(C=64, D=40, S=512, bits=4, padding=64, sbeams=2, beams=2, seed=3)
    got = engine_run(case)
    want = _plan_out(case)
    np.testing.assert_array_equal(case.valid(got).view(np.uint32),
                                  case.valid(want).view(np.uint32))
