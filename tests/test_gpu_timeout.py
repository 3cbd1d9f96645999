"""The bounded-wait failure path of the tensor-core kernel, without a GPU fault.

Every wait of ``mixed_kernel`` on a pipeline barrier is bounded.  The test
hook ``vl1_test_set_wait_fault`` shortens the bound (5 ms) and has one producer warp
of the first CTA withhold its first arrival: a barrier that nothing
completes, so the issuer's wait runs out.  The kernel must then let its
issued copies and MMAs finish, free its TMEM, write no results for that CTA,
report ``VL1_E_TIMEOUT`` in the status word (mapped to ``VL1TimeoutError``),
and leave the device, the plan and the schedule usable: the next call on the
same plan and schedule is correct.
"""

import ctypes as C

import numpy as np
import pytest

from helpers import LAP2, LAP3, oracle_eval, oracle_for_workload, plan_and_view, rel_l2
from volumential_gb300 import _lib
from volumential_gb300 import workloads as W
from volumential_gb300.batch import BatchProblem, MixedBatch, problem_arrays
from volumential_gb300.batched import get_schedule
from volumential_gb300.plan import as_device_tensor

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-9
WAIT_LIMIT_US = 5000   # a wait gives up after 5 ms


class _WaitFault:
    def __enter__(self):
        _lib.check(_lib.lib().vl1_test_set_wait_fault(WAIT_LIMIT_US, 1), "vl1_test_set_wait_fault")

    def __exit__(self, *exc):
        _lib.check(_lib.lib().vl1_test_set_wait_fault(0, 0), "vl1_test_set_wait_fault")


def _eval(lib, plan, view, sched, coefs, out, nrhs, stream):
    _lib.check(lib.vl1_eval_mixed(plan.handle, C.byref(view), C.byref(sched.c_struct),
                                  coefs.data_ptr(), nrhs, out.data_ptr(),
                                  sched.workspace.data_ptr(), sched.workspace.numel(),
                                  C.c_void_p(stream)), "vl1_eval_mixed")


@pytest.mark.parametrize("cap", [None, 3])   # 3: tiles split over several CTAs
def test_timeout_is_reported_and_the_next_call_is_correct(cuda, cap):
    torch = cuda
    w = W.uniform_workload("timeout", 3, 3, 4, seed=71, nrhs=2)   # 8 tiles
    plan, view, keep = plan_and_view(w)
    stream = torch.cuda.current_stream().cuda_stream
    sched = get_schedule(plan, view, keep, w.nrhs, stream, max_keys_per_item=cap)
    assert sched.n_tiles > 1
    if cap is not None:
        assert sched.n_splits > 0
    coefs = as_device_tensor(np.ascontiguousarray(w.coefs))
    lib = _lib.lib()
    plan.read_status(stream, reset=True)

    out = torch.full((w.nrhs, w.n_points), float("nan"), dtype=torch.float64, device="cuda")
    with _WaitFault():
        _eval(lib, plan, view, sched, coefs, out, w.nrhs, stream)
        torch.cuda.synchronize()
    with pytest.raises(_lib.VL1TimeoutError, match="bounded device wait"):
        plan.raise_on_status(stream)
    got = out.cpu().numpy()
    assert np.isnan(got).any()          # the timed-out CTA wrote nothing
    assert np.isfinite(got).any()       # the others completed

    # the same plan and schedule again, without the hook: correct and clean
    out2 = torch.full_like(out, float("nan"))
    _eval(lib, plan, view, sched, coefs, out2, w.nrhs, stream)
    plan.raise_on_status(stream)
    assert int(sched.split_counters.abs().max()) == 0
    prob = oracle_for_workload(w, LAP3)
    got2 = out2.cpu().numpy()
    for r in range(w.nrhs):
        assert rel_l2(got2[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED


def test_timeout_in_a_persistent_batch_launch(cuda):
    torch = cuda
    ws = [W.uniform_workload("tb2", 2, 4, 4, seed=72, nrhs=2),
          W.uniform_workload("tb3", 3, 3, 3, seed=73, nrhs=1)]
    probs = []
    for w in ws:
        plan, view, keep = problem_arrays(w)
        coefs = as_device_tensor(np.ascontiguousarray(w.coefs))
        out = torch.full((w.nrhs, w.n_points), float("nan"), dtype=torch.float64,
                         device="cuda")
        probs.append(BatchProblem(plan, view, keep, coefs, out, w.nrhs))
    batch = MixedBatch(probs, max_keys_per_item=2)
    for p in probs:
        p.plan.read_status(reset=True)
    with _WaitFault():
        batch.eval()
        torch.cuda.synchronize()
    with pytest.raises(_lib.VL1TimeoutError):
        batch.raise_on_status()
    for p in probs:
        p.plan.read_status(reset=True)   # the other plans' words as well
        p.out.fill_(float("nan"))
    batch.eval()
    batch.raise_on_status()
    for w, p, pol in zip(ws, probs, (LAP2, LAP3)):
        prob = oracle_for_workload(w, pol)
        got = p.out.cpu().numpy()
        for r in range(w.nrhs):
            assert rel_l2(got[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED
