"""Tiles split over several CTAs (key ranges) in the tensor-core path.

A tile whose target boxes need many (table level, case) keys is split into
work items; each item stores exact partial sums and the last one to finish adds
them in slot order.  The split result must match the oracle within the
mixed-precision tolerance and the unsplit result to rounding of the FP32 tails
(the integer parts are exact in both), and repeated calls must give identical
results (the split counters return to zero after every call).
"""

import numpy as np
import pytest

from helpers import FIXED, LAP2, LAP3, oracle_eval, oracle_for_workload, plan_and_view, rel_l2
from volumential_gb300 import workloads as W
from volumential_gb300.batched import eval_mixed, get_schedule
from volumential_gb300.kernels import HelmholtzKernel
from volumential_gb300.plan import as_device_tensor

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-9
TOL_SPLIT = 2e-11


def _run(torch, w, cap):
    plan, view, keep = plan_and_view(w)
    stream = torch.cuda.current_stream().cuda_stream
    nrhs = w.coefs.shape[0]
    coefs = as_device_tensor(np.ascontiguousarray(w.coefs))
    odt = torch.complex128 if plan.complex_table else torch.float64
    outs = []
    for _ in range(2):
        out = torch.full((nrhs, w.n_points), float("nan"), dtype=odt, device="cuda")
        eval_mixed(plan, view, coefs, out, stream=stream, nrhs=nrhs, keep=keep,
                   max_keys_per_item=cap)
        plan.raise_on_status(stream)
        outs.append(out.cpu().numpy())
    sched = get_schedule(plan, view, keep, nrhs, stream, cap)
    assert np.array_equal(outs[0], outs[1])
    return outs[0], sched


@pytest.mark.parametrize("cap", [1, 3, 7])
def test_split_adaptive_3d_matches_unsplit_and_oracle(cuda, cap):
    torch = cuda
    w = W.adaptive_workload("sp3", 3, 4, tol=3e-2, max_level=5, min_level=2, seed=51)
    whole, s0 = _run(torch, w, 1 << 30)
    assert s0.n_splits == 0
    split, s1 = _run(torch, w, cap)
    assert s1.n_splits > 0 and s1.max_keys_per_item <= cap
    # the FP32 tail sums (whose last density plane carries fractional bits)
    # round differently over different key ranges; the exact parts agree
    assert rel_l2(split[0], whole[0]) <= TOL_SPLIT
    prob = oracle_for_workload(w, LAP3)
    assert rel_l2(split[0], oracle_eval(prob, w, w.coefs[0])) <= TOL_MIXED


def test_split_two_column_chunks(cuda):
    # 3D q = 5: 125 target points -> two 64-column chunks per tile, each chunk
    # with its own split counter
    torch = cuda
    w = W.uniform_workload("sp5", 3, 2, 5, seed=52, nrhs=2)
    split, s1 = _run(torch, w, 2)
    assert s1.n_splits > 0
    prob = oracle_for_workload(w, LAP3)
    for r in range(2):
        assert rel_l2(split[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED


def test_split_complex_table_many_rhs(cuda):
    torch = cuda
    w = W.uniform_workload("sph", 2, 4, 5, seed=53, kernel=HelmholtzKernel(2),
                           complex_table=True, nrhs=3)
    w.tables = W.synthetic_tables(2, 5, w.kernel, seed=7, complex_values=True,
                                  source_box_extent=w.tree.root_extent / 16)
    split, s1 = _run(torch, w, 2)
    assert s1.n_splits > 0
    prob = oracle_for_workload(w, FIXED)
    for r in range(3):
        assert rel_l2(split[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED


def test_split_2d_uniform(cuda):
    torch = cuda
    w = W.uniform_workload("sp2", 2, 4, 4, seed=54, nrhs=2)
    split, s1 = _run(torch, w, 2)
    prob = oracle_for_workload(w, LAP2)
    for r in range(2):
        assert rel_l2(split[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED
