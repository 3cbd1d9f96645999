"""The mixed path's schedule built on the device (``vl1_schedule_build_*``).

Its box order is restated here in numpy (keys ranked by frequency, rarest
first, ties by key id; boxes sorted stably by their key sets read as bit
strings with the rarest key most significant); given that order, every array
of the schedule must equal the host builder's (``MixedSchedule.tile_schedule``)
exactly, and evaluations with the device schedule and with the host's greedy
packing must both match the FP64 oracle within the mixed tolerance.
"""

import numpy as np
import pytest

from helpers import LAP2, LAP3, oracle_eval, oracle_for_workload, plan_and_view, rel_l2
from volumential_gb300 import _lib
from volumential_gb300 import workloads as W
from volumential_gb300.batched import MixedSchedule, eval_mixed, get_schedule
from volumential_gb300.plan import as_device_tensor

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-9


def _device_order(keys, starts, n_tb, K):
    tb_of_pair = np.repeat(np.arange(n_tb), np.diff(starts))
    mask = np.zeros((n_tb, K), dtype=bool)
    mask[tb_of_pair, keys] = True
    by = np.argsort(np.bincount(keys, minlength=K), kind="stable")   # rarest first
    cols = mask[:, by]
    return np.lexsort(tuple(cols[:, r] for r in range(K - 1, -1, -1)))


CASES = [
    ("u2", lambda: W.uniform_workload("s_u2", 2, 4, 4, seed=501), LAP2, 1),
    ("u3", lambda: W.uniform_workload("s_u3", 3, 2, 3, seed=502, nrhs=3), LAP3, 3),
    ("ad3", lambda: W.adaptive_workload("s_ad3", 3, 3, tol=3e-2, max_level=5, min_level=2,
                                        seed=503), LAP3, 1),
    ("ad2_rhs130", lambda: W.adaptive_workload("s_ad2", 2, 3, tol=1e-3, max_level=6,
                                               min_level=2, seed=504, n_terms=8,
                                               width_range=(0.02, 0.1)), LAP2, 130),
]


@pytest.mark.parametrize("name,make,policy,nrhs", CASES, ids=[c[0] for c in CASES])
def test_device_schedule_equals_host_restatement(cuda, name, make, policy, nrhs):
    torch = cuda
    w = make()
    plan, view, keep = plan_and_view(w)
    stream = torch.cuda.current_stream().cuda_stream
    dev = MixedSchedule(plan, view, keep, nrhs, stream, packing="device", workspace=False)
    tr = w.traversal
    K = plan.n_tables * plan.n_cases
    keys = torch.empty(max(tr.nnz, 1), dtype=torch.int32, device="cuda")
    import ctypes as C
    _lib.check(_lib.lib().vl1_classify_pairs(plan.handle, C.byref(view), keys.data_ptr(),
                                             C.c_void_p(stream)), "vl1_classify_pairs")
    keys = keys[:tr.nnz].cpu().numpy().astype(np.int64)
    starts = np.asarray(tr.neighbor_source_boxes_starts, dtype=np.int64)
    lists = np.asarray(tr.neighbor_source_boxes_lists, dtype=np.int64)
    order = _device_order(keys, starts, len(tr.target_boxes), K)
    rows, key_start, key_ids, xrow = MixedSchedule.tile_schedule(
        keys, starts, lists, len(tr.target_boxes), K, nrhs, order=order)
    assert dev.n_tiles == len(rows) and dev.n_tile_keys == len(key_ids)
    assert np.array_equal(dev.key_start_np, key_start)
    assert np.array_equal(dev.tile_rows.cpu().numpy().reshape(-1, 128), rows)
    assert np.array_equal(dev.tile_key_start.cpu().numpy(), key_start)
    assert np.array_equal(dev.key_ids[:len(key_ids)].cpu().numpy(), key_ids)
    assert np.array_equal(dev.key_xrow[:xrow.size].cpu().numpy().reshape(-1, 128), xrow)


@pytest.mark.parametrize("packing", ["device", "greedy"])
def test_both_packings_match_the_oracle(cuda, packing):
    torch = cuda
    w = W.adaptive_workload("s_pk", 3, 4, tol=3e-2, max_level=5, min_level=2, seed=505,
                            nrhs=2)
    plan, view, keep = plan_and_view(w)
    stream = torch.cuda.current_stream().cuda_stream
    sched = get_schedule(plan, view, keep, w.nrhs, stream, packing=packing)
    assert sched.packing == packing
    coefs = as_device_tensor(np.ascontiguousarray(w.coefs)).reshape(-1)
    out = torch.empty_like(coefs)
    eval_mixed(plan, view, coefs, out, stream=stream, nrhs=w.nrhs, keep=keep)
    plan.raise_on_status(stream)
    got = out.view(w.nrhs, -1).cpu().numpy()
    prob = oracle_for_workload(w, LAP3)
    for r in range(w.nrhs):
        assert rel_l2(got[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED


def test_duplicate_mode_ids_are_rejected_by_the_device_builder(cuda):
    torch = cuda
    w = W.uniform_workload("s_dup", 2, 2, 3, seed=506)
    plan, view, keep = plan_and_view(w)
    bad = keep["smode"].clone()
    bad[1] = bad[0]
    keep2 = dict(keep, smode=bad)
    view.source_mode_ids = bad.data_ptr()
    try:
        with pytest.raises(ValueError, match="distinct source mode ids"):
            MixedSchedule(plan, view, keep2, 1, torch.cuda.current_stream().cuda_stream,
                          packing="device", workspace=False)
    finally:
        view.source_mode_ids = keep["smode"].data_ptr()
