"""The allocation-free entry point ``vl1_eval_mixed_noalloc``.

Some callers of this library cannot allocate device memory at evaluation time:
a host solver that owns every byte of device memory through its own pool, or a
latency-critical loop that cannot afford cudaMalloc's device synchronisation.
For them the tensor-core evaluation has a variant whose scratch lives in a
fixed array inside the library.  This test calls it through the C ABI twice in
a row and checks each result against ``vl1_eval_mixed`` (caller-provided
workspace) on the same inputs and against the FP64 oracle, within the
mixed-precision tolerance, and that the calls allocate no device memory
(the driver's free-memory count and torch's allocator do not move).  It
also runs a complex-valued (Helmholtz) table, a large problem followed by a
smaller one (every scratch value a call reads must be its own), and checks
that a problem larger than the fixed array is refused cleanly.

The file name makes pytest collect it last.
"""

import ctypes as C

import numpy as np
import pytest

from helpers import FIXED, LAP2, LAP3, oracle_eval, oracle_for_workload, rel_l2, wrangler_for
from volumential_gb300 import _lib
from volumential_gb300 import workloads as W
from volumential_gb300.kernels import HelmholtzKernel
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


def _helmholtz_workload():
    w = W.uniform_workload("noalloc_helm", 2, 3, 4, seed=45, nrhs=2,
                           kernel=HelmholtzKernel(2), complex_table=True)
    w.tables = W.synthetic_tables(2, 4, w.kernel, seed=46, complex_values=True,
                                  source_box_extent=w.tree.root_extent / 8)
    return w, FIXED


CASES = {
    "lap2d_q4_3rhs": lambda: (W.uniform_workload("noalloc", 2, 4, 4, seed=43, nrhs=3), LAP2),
    "lap3d_q4": lambda: (W.uniform_workload("noalloc", 3, 2, 4, seed=44, nrhs=1), LAP3),
    "helm2d_complex_table": _helmholtz_workload,
}


class _Problem:
    """Plan, tree, schedule, coefficients, the workspace entry point's result
    and the oracle's result of one workload."""

    def __init__(self, torch, w, policy):
        self.w = w
        self.plan, self.view, self.keep = _setup(w)
        self.stream = torch.cuda.current_stream().cuda_stream
        self.nrhs = w.nrhs
        self.sched = get_schedule(self.plan, self.view, self.keep, self.nrhs, self.stream)
        self.coefs = as_device_tensor(np.ascontiguousarray(w.coefs))
        self.odt = torch.complex128 if self.plan.complex_table else torch.float64
        lib = _lib.lib()
        need = lib.vl1_mixed_workspace_bytes(self.plan.handle, C.byref(self.view), self.nrhs)
        assert 0 < need <= _lib.VL1_NOALLOC_SCRATCH_BYTES
        ref = torch.zeros((self.nrhs, w.n_points), dtype=self.odt, device="cuda")
        _lib.check(lib.vl1_eval_mixed(self.plan.handle, C.byref(self.view),
                                      C.byref(self.sched.c_struct), self.coefs.data_ptr(),
                                      self.nrhs, ref.data_ptr(),
                                      self.sched.workspace.data_ptr(),
                                      self.sched.workspace.numel(), C.c_void_p(self.stream)),
                   "vl1_eval_mixed")
        self.plan.raise_on_status(self.stream)
        self.ref = ref.cpu().numpy()
        assert np.all(np.isfinite(self.ref)) and np.linalg.norm(self.ref) > 0
        prob = oracle_for_workload(w, policy)
        self.oracle = [oracle_eval(prob, w, w.coefs[r]) for r in range(self.nrhs)]

    def noalloc(self, out):
        _lib.check(_lib.lib().vl1_eval_mixed_noalloc(
            self.plan.handle, C.byref(self.view), C.byref(self.sched.c_struct),
            self.coefs.data_ptr(), self.nrhs, out.data_ptr(), C.c_void_p(self.stream)),
            "vl1_eval_mixed_noalloc")
        self.plan.raise_on_status(self.stream)

    def check(self, got):
        for r in range(self.nrhs):
            assert rel_l2(got[r], self.ref[r]) <= TOL_MIXED
            assert rel_l2(got[r], self.oracle[r]) <= TOL_MIXED


@pytest.mark.parametrize("case", sorted(CASES))
def test_noalloc_matches_workspace_entry_point_twice(cuda, case):
    torch = cuda
    p = _Problem(torch, *CASES[case]())
    outs = [torch.full((p.nrhs, p.w.n_points), float("nan"), dtype=p.odt, device="cuda")
            for _ in range(2)]
    p.noalloc(outs[0])                 # first call: the scratch address is looked up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    alloc0 = torch.cuda.memory_allocated()
    for out in outs:
        p.noalloc(out)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0      # no device allocation
        assert torch.cuda.memory_allocated() == alloc0
        p.check(out.cpu().numpy())


def test_noalloc_large_then_small_problem(cuda):
    torch = cuda
    big = _Problem(torch, W.uniform_workload("noalloc_big3", 3, 3, 4, seed=48, nrhs=2), LAP3)
    small = _Problem(torch, W.uniform_workload("noalloc_small2", 2, 3, 3, seed=49, nrhs=1),
                     LAP2)
    for p in (big, small, big, small):
        out = torch.full((p.nrhs, p.w.n_points), float("nan"), dtype=p.odt, device="cuda")
        p.noalloc(out)
        p.check(out.cpu().numpy())


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
