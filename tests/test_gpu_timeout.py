"""The device-side timeout path, driven without a fault.

Every wait of a tile kernel for a staged copy is bounded.  When one runs out
the CTA records kStatusTimeout in the plan's status word, lets its copies in
flight land (the drain keeps its own 50 ms limit) and returns; the host then
reports DD_ERR_TIMEOUT and the context stays usable.  Here the plan's wait
limit is set to 1 ns (dd_plan_set_wait_limit), which makes the waits run out
on copies that have not landed yet: the run must report DD_ERR_TIMEOUT, and
the same plan with the default limit restored must then give the oracle's
output (include/Dedispersion.hpp:70-109), for every kernel family (the
shared-partial-sum tile, the direct swar8 tile, the scalar tiles for 16-bit
and float input, the TMEM-window tile for float input).  The reference reports OpenCL errors to its caller in the
same way (src/DedispersionTuning.cpp:396-409).
"""
import numpy as np
import pytest

import dedispersion_gb300 as dd
from dedispersion_gb300 import _abi

from helpers import single_case

pytestmark = pytest.mark.gpu


def _kernel(name):
    return next(k.index for k in dd.kernels() if k.name == name)


CASES = [
    ("shared8 default", 8, None),
    ("swar8", 8, "swar8_i4_d4_w8_c16_vkUnpackPermuteMad"),
    ("scalar16", 16, "scalar16_i8_d4_w8_c16"),
    ("scalar32", 32, "scalar32_i8_d8_w4_c16"),
    ("tmem32", 32, "tmem32_t16_d64"),
]


@pytest.mark.parametrize("label,bits,kernel", CASES, ids=[c[0] for c in CASES])
def test_wait_timeout_reports_and_plan_recovers(gpu, oracle, label, bits, kernel):
    torch = pytest.importorskip("torch")
    case = single_case(C=256, D=128, S=2048, bits=bits, padding=128, zap=0.05, seed=71,
                       dist="uniform" if bits <= 16 else "gaussian")
    plan = dd.Plan(case.obs, dd.DD_SINGLE_STEP, bits, case.padding,
                   kernel=None if kernel is None else _kernel(kernel))
    plan.setShifts(case.shifts)
    plan.setZappedChannels(case.zapped)
    plan.setBeamMapping(case.mapping)
    if kernel is None:
        assert plan.conf().getNrItemsD2() == 8, "the default plan runs the shared tile"
    d_in = torch.from_numpy(case.inp).cuda()
    d_out = torch.zeros(case.out_elems, dtype=torch.float32, device="cuda")
    plan.setWaitLimit(1)
    plan.run(d_in, d_out)
    with pytest.raises(dd.DedispersionError) as e:
        plan.check()
    assert e.value.status == _abi.DD_ERR_TIMEOUT
    assert "bounded wait" in str(e.value)
    # the status word was reset by the check; the context still works
    plan.setWaitLimit(0)
    plan.run(d_in, d_out)
    plan.check()
    want = case.output()
    oracle.dedispersion(case.obs.c, case.zapped, case.mapping, case.inp, want, case.shifts,
                        case.padding, bits)
    got = case.valid(d_out.cpu().numpy())
    assert np.array_equal(got.view(np.uint32), case.valid(want).view(np.uint32))
    plan.close()
