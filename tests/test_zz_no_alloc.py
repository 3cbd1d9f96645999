"""The allocation-free entry point ``vl1_eval_mixed_noalloc``.

Some callers of this library cannot allocate device memory at evaluation time:
a host solver that owns every byte of device memory through its own pool, or a
latency-critical loop that cannot afford cudaMalloc's device synchronisation.
For them the tensor-core evaluation has a variant whose scratch lives in a
fixed array inside the library.  This test calls it through the C ABI twice in
a row and checks each result against ``vl1_eval_mixed`` (caller-provided
workspace) on the same inputs, within the mixed-precision tolerance; it also
checks that a problem larger than the fixed array is refused cleanly.

The file name makes pytest collect it last.
"""

import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2, wrangler_for
from volumential_gb300 import _lib
from volumential_gb300 import workloads as W
from volumential_gb300.batched import get_schedule
from volumential_gb300.plan import as_device_tensor, tree_view_from_arrays

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-9
TREE_KEYS = ("target_boxes", "neighbor_source_boxes_starts", "neighbor_source_boxes_lists",
             "box_centers", "box_levels", "box_source_starts", "box_source_counts_nonchild",
             "box_target_starts", "box_target_counts_nonchild", "source_mode_ids",
             "target_point_ids")


def _setup(w):
    wr = wrangler_for(w)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, None)
    plan = nf.get_plan(
        table_data_combined=kw["table_data_combined"],
        mode_nmlz_combined=kw["mode_nmlz_combined"], case_indices=kw["case_indices"],
        encoding_base=kw["encoding_base"], encoding_shift=kw["encoding_shift"],
        table_root_extent=kw["table_root_extent"],
        table_starting_level=kw["table_starting_level"],
        **{n: kw[n] for n in kw if n.startswith("arithmetic_")})
    view, keep = tree_view_from_arrays(root_extent=kw["root_extent"],
                                       **{k: kw[k] for k in TREE_KEYS})
    return plan, view, keep


@pytest.mark.parametrize("dim,level,q,nrhs", [(2, 4, 4, 3), (3, 2, 4, 1)])
def test_noalloc_matches_workspace_entry_point_twice(cuda, dim, level, q, nrhs):
    torch = cuda
    w = W.uniform_workload("noalloc", dim, level, q, seed=41 + dim, nrhs=nrhs)
    plan, view, keep = _setup(w)
    stream = torch.cuda.current_stream().cuda_stream
    sched = get_schedule(plan, view, keep, nrhs, stream)
    coefs = as_device_tensor(np.ascontiguousarray(w.coefs))
    n = w.n_points
    lib = _lib.lib()
    need = lib.vl1_mixed_workspace_bytes(plan.handle, C.byref(view), nrhs)
    assert 0 < need <= _lib.VL1_NOALLOC_SCRATCH_BYTES

    ref = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
    _lib.check(lib.vl1_eval_mixed(plan.handle, C.byref(view), C.byref(sched.c_struct),
                                  coefs.data_ptr(), nrhs, ref.data_ptr(),
                                  sched.workspace.data_ptr(), sched.workspace.numel(),
                                  C.c_void_p(stream)), "vl1_eval_mixed")
    plan.raise_on_status(stream)
    ref_h = ref.cpu().numpy()
    assert np.all(np.isfinite(ref_h)) and np.linalg.norm(ref_h) > 0

    for _ in range(2):
        out = torch.full((nrhs, n), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(lib.vl1_eval_mixed_noalloc(plan.handle, C.byref(view),
                                              C.byref(sched.c_struct), coefs.data_ptr(),
                                              nrhs, out.data_ptr(), C.c_void_p(stream)),
                   "vl1_eval_mixed_noalloc")
        plan.raise_on_status(stream)
        got = out.cpu().numpy()
        for r in range(nrhs):
            assert rel_l2(got[r], ref_h[r]) <= TOL_MIXED


def test_noalloc_refuses_problems_above_its_fixed_scratch(cuda):
    torch = cuda
    w = W.uniform_workload("noalloc_big", 2, 3, 2, seed=47, nrhs=1)
    plan, view, keep = _setup(w)
    lib = _lib.lib()
    nrhs = 1
    while lib.vl1_mixed_workspace_bytes(plan.handle, C.byref(view), nrhs) <= \
            _lib.VL1_NOALLOC_SCRATCH_BYTES:
        nrhs *= 2
    n = w.n_points
    coefs = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
    out = torch.zeros((nrhs, n), dtype=torch.float64, device="cuda")
    sched = _lib.MixedSchedule()  # never read: the size check comes first
    st = lib.vl1_eval_mixed_noalloc(plan.handle, C.byref(view), C.byref(sched),
                                    coefs.data_ptr(), nrhs, out.data_ptr(),
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _lib.VL1_E_ARG
    assert b"fixed" in lib.vl1_last_error_string()
    assert float(out.abs().max()) == 0.0
