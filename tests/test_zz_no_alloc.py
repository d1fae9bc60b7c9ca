"""dd_dedispersion_noalloc: single-step dedispersion for callers that cannot
call cudaMalloc where they dedisperse (a real-time loop that must not block
on an allocation, or a framework that owns all device memory in its own
capped pool).  Its working tables live in a fixed device array inside the
library, so this test checks that two consecutive calls through the C ABI --
the second with a different shape, mask and input width, so stale tables from
the first would show -- give exactly what the plan entry point gives, and that
a request beyond the array's limit is refused with a clear error.

The file sorts last so that a run stopping at the first failure has run every
other test before this one.
"""
import ctypes as C

import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import _abi

from helpers import single_case

pytestmark = pytest.mark.gpu

U32P = C.POINTER(C.c_uint32)
F32P = C.POINTER(C.c_float)


def plan_output(torch, case, d_in):
    out = torch.zeros(case.out_elems, dtype=torch.float32, device="cuda")
    plan = dd.Plan(case.obs, dd.DD_SINGLE_STEP, case.bits, case.padding)
    plan.setShifts(case.shifts)
    plan.setZappedChannels(case.zapped)
    plan.setBeamMapping(case.mapping)
    plan.run(d_in, out)
    plan.check()
    plan.close()
    return out.cpu().numpy()


def noalloc(case, d_in, d_out, stream=0):
    return _abi.lib().dd_dedispersion_noalloc(
        C.byref(case.obs.c), case.zapped.ctypes.data_as(U32P), case.mapping.ctypes.data_as(U32P),
        C.c_void_p(d_in.data_ptr()), C.cast(C.c_void_p(d_out.data_ptr()), F32P),
        case.shifts.ctypes.data_as(F32P), case.padding, case.bits, C.c_void_p(stream))


def test_noalloc_matches_plan_on_two_calls_in_a_row(gpu):
    torch = pytest.importorskip("torch")
    cases = [
        single_case(C=300, D=70, S=1500, bits=8, padding=64, beams=2, sbeams=2, zap=0.05,
                    seed=31, dist="gaussian", sigma=40.0),
        single_case(C=130, D=45, S=900, bits=4, padding=16, beams=3, sbeams=3, zap=0.2, seed=32),
    ]
    stream = torch.cuda.Stream()
    for case in cases:
        d_in = torch.from_numpy(case.inp).cuda()
        want = plan_output(torch, case, d_in)
        # garbage in the output buffer must be overwritten wherever it is defined
        d_out = torch.full((case.out_elems,), -7.0, dtype=torch.float32, device="cuda")
        # the fill and the copy above ran on torch's current stream
        stream.wait_stream(torch.cuda.current_stream())
        rc = noalloc(case, d_in, d_out, stream.cuda_stream)
        assert rc == 0, _abi.lib().dd_last_error().decode()
        got = d_out.cpu().numpy()
        g, w = case.valid(got), case.valid(want)
        # integer input: the tolerance is exact equality
        assert np.array_equal(g.view(np.uint32), w.view(np.uint32))


def test_noalloc_rejects_requests_beyond_its_limit(gpu):
    torch = pytest.importorskip("torch")
    case = single_case(C=64, D=8, S=64, bits=8, padding=0, zap=0.0, seed=33)
    big = case.obs.copy()
    big.setNrSynthesizedBeams(5000)
    mapping = np.zeros(5000 * 64, np.uint32)
    d_in = torch.from_numpy(case.inp).cuda()
    d_out = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = _abi.lib().dd_dedispersion_noalloc(
        C.byref(big.c), case.zapped.ctypes.data_as(U32P), mapping.ctypes.data_as(U32P),
        C.c_void_p(d_in.data_ptr()), C.cast(C.c_void_p(d_out.data_ptr()), F32P),
        case.shifts.ctypes.data_as(F32P), 0, 8, None)
    assert rc == _abi.DD_ERR_UNSUPPORTED
    assert "no-alloc limit" in _abi.lib().dd_last_error().decode()
    # under the beam limit, over the 61440 live rows: 16 beams x 4096 channels
    wide = single_case(C=4096, D=8, S=64, bits=8, padding=0, zap=0.0, seed=34)
    many = wide.obs.copy()
    many.setNrSynthesizedBeams(16)
    mapping = np.zeros(16 * 4096, np.uint32)
    rc = _abi.lib().dd_dedispersion_noalloc(
        C.byref(many.c), wide.zapped.ctypes.data_as(U32P), mapping.ctypes.data_as(U32P),
        C.c_void_p(d_in.data_ptr()), C.cast(C.c_void_p(d_out.data_ptr()), F32P),
        wide.shifts.ctypes.data_as(F32P), 0, 8, None)
    assert rc == _abi.DD_ERR_UNSUPPORTED
    msg = _abi.lib().dd_last_error().decode()
    assert "65536 live rows" in msg and "no-alloc limit of 61440" in msg
