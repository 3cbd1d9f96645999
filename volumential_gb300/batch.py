"""Batches of list-1 problems evaluated together on the tensor cores.

Many right-hand sides and many trees of uneven depth and quadrature order go
through one set of launches: batched preparation kernels, then one persistent
tensor-core launch per kernel shape in which every CTA takes the next
(problem, tile, column chunk) work item from a queue, longest first.  The
launches of one evaluation allocate nothing and do not synchronise the host,
so :meth:`MixedBatch.capture` records them in a CUDA graph that
:meth:`MixedBatch.replay` re-runs on the current coefficients.

The reference evaluates one output kernel and tree per ``NearFieldFromCSR``
call (``expansion_wrangler_fpnd.py:3417-3442``); a batch is the many-problem
form of that call, with the same per-problem inputs and outputs.
"""

from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib
from .batched import MixedSchedule, get_schedule

__all__ = ["BatchProblem", "MixedBatch", "autotune_batch", "plan_for", "problem_arrays",
           "tree_arrays"]

TREE_KEYS = ("target_boxes", "neighbor_source_boxes_starts", "neighbor_source_boxes_lists",
             "box_centers", "box_levels", "box_source_starts", "box_source_counts_nonchild",
             "box_target_starts", "box_target_counts_nonchild", "source_mode_ids",
             "target_point_ids")


class BatchProblem:
    """One problem of a batch: a plan, a tree view (device arrays kept alive
    in ``keep``), device coefficients [nrhs, N] (float64) and the device
    result buffer of the plan's output dtype."""

    def __init__(self, plan, view, keep, coefs, out, nrhs):
        self.plan, self.view, self.keep = plan, view, keep
        self.coefs, self.out, self.nrhs = coefs, out, int(nrhs)


def _plan_kwargs(workload):
    from .expansion_wrangler_fpnd import (FPNDExpansionWrangler,
                                          FPNDTreeIndependentDataForWrangler)

    w = workload
    ti = FPNDTreeIndependentDataForWrangler(target_kernels=[w.kernel])
    dtype = np.complex128 if w.kernel.is_complex_valued else np.float64
    wr = FPNDExpansionWrangler(ti, w.traversal, w.tables, dtype=dtype, quad_order=w.q)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, None)
    return nf, kw


def _plan_from(nf, kw, cache):
    return nf.get_plan(
        table_data_combined=kw["table_data_combined"],
        mode_nmlz_combined=kw["mode_nmlz_combined"], case_indices=kw["case_indices"],
        encoding_base=kw["encoding_base"], encoding_shift=kw["encoding_shift"],
        table_root_extent=kw["table_root_extent"],
        table_starting_level=kw["table_starting_level"], cache=cache,
        **{n: kw[n] for n in kw if n.startswith("arithmetic_")})


def _view_from(kw):
    from .plan import as_device_tensor, tree_view_from_arrays

    return tree_view_from_arrays(root_extent=kw["root_extent"],
                                 **{k: as_device_tensor(kw[k]) for k in TREE_KEYS})


def problem_arrays(workload, plan=None, cache=True):
    """(plan, view, keep) of a workload through the FPND wrangler's argument
    assembly; ``plan`` reuses an existing plan of the same table set;
    ``cache=False`` makes a new plan owned by the caller (outside the
    process-wide plan cache, which destroys its oldest plans)."""
    nf, kw = _plan_kwargs(workload)
    if plan is None:
        plan = _plan_from(nf, kw, cache)
    view, keep = _view_from(kw)
    return plan, view, keep


def plan_for(workload, cache=True):
    """The device plan of a workload's table set (as ``problem_arrays``)."""
    nf, kw = _plan_kwargs(workload)
    return _plan_from(nf, kw, cache)


def tree_arrays(workload):
    """(view, keep) of a workload's tree in the FPND wrangler's argument
    layout (expansion_wrangler_fpnd.py:3402-3424: sources are the targets,
    box-local mode ids), without building its tables' payload."""
    from .expansion_wrangler_fpnd import (_compute_box_local_ids,
                                          _validate_table_box_particle_layout)

    w = workload
    tree, tr = w.tree, w.traversal
    nq = w.q ** w.dim
    _validate_table_box_particle_layout(tree, tr.target_boxes, tr.neighbor_source_boxes_lists,
                                        nq)
    local = _compute_box_local_ids(tree, nq)
    counts = np.asarray(tree.box_target_counts_nonchild).astype(np.int32)
    kw = dict(target_boxes=tr.target_boxes,
              neighbor_source_boxes_starts=tr.neighbor_source_boxes_starts,
              neighbor_source_boxes_lists=tr.neighbor_source_boxes_lists,
              box_centers=tree.box_centers, box_levels=tree.box_levels,
              box_source_starts=tree.box_target_starts, box_source_counts_nonchild=counts,
              box_target_starts=tree.box_target_starts, box_target_counts_nonchild=counts,
              source_mode_ids=local, target_point_ids=local, root_extent=tree.root_extent)
    return _view_from(kw)


class MixedBatch:
    """A fixed set of problems evaluated by one ``vl1_batch_eval`` call.

    ``max_keys_per_item`` caps the keys of one work item (long tiles are split
    over several CTAs; ``None`` lets each problem's schedule choose);
    ``ctas_per_launch`` sets the persistent CTAs per kernel shape (0: one per
    SM).  Coefficient and result tensors are used in place: write new
    densities into ``problem.coefs`` and call :meth:`eval` or :meth:`replay`.
    """

    def __init__(self, problems, *, max_keys_per_item=None, ctas_per_launch=0, stream=None):
        import torch

        self.problems = list(problems)
        if not self.problems:
            raise ValueError("a batch needs at least one problem")
        self._lib = _lib.lib()
        self.handle = None
        sh = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        self.schedules = []
        arr = (_lib.BatchProblem * len(self.problems))()
        used = set()
        for i, p in enumerate(self.problems):
            if p.coefs.dtype != torch.float64 or not p.coefs.is_contiguous():
                raise TypeError("batch coefficients must be contiguous float64 tensors")
            if p.coefs.numel() != p.nrhs * int(p.view.n_particles):
                raise ValueError(f"problem {i}: coefficients must hold nrhs * N values")
            sched = get_schedule(p.plan, p.view, p.keep, p.nrhs, sh, max_keys_per_item)
            if id(sched) in used and sched.n_splits > 0:
                # problems of one plan, tree and rhs count share the cached
                # schedule; each needs its own split scratch
                sched = MixedSchedule(p.plan, p.view, p.keep, p.nrhs, sh, max_keys_per_item,
                                      base=sched, workspace=False)
            used.add(id(sched))
            self.schedules.append(sched)
            arr[i].plan = p.plan.handle
            arr[i].tree = C.cast(C.pointer(p.view), C.c_void_p)
            arr[i].schedule = C.cast(C.pointer(sched.c_struct), C.c_void_p)
            arr[i].coefs = p.coefs.data_ptr()
            arr[i].nrhs = p.nrhs
            arr[i].result = p.out.data_ptr()
            arr[i].host_items = sched.items_np.ctypes.data
        self._arr = arr
        opt = _lib.BatchOptions(int(ctas_per_launch), 0)
        handle = C.c_void_p()
        torch.cuda.current_stream().synchronize()
        _lib.check(self._lib.vl1_batch_create(len(self.problems), arr, C.byref(opt),
                                              C.byref(handle)), "vl1_batch_create")
        self.handle = handle
        self.graph = None
        self.max_keys_per_item = max_keys_per_item
        self.ctas_per_launch = int(ctas_per_launch)

    @property
    def device_bytes(self):
        return int(self._lib.vl1_batch_device_bytes(self.handle))

    @property
    def kernel_launches(self):
        """Kernels one evaluation launches."""
        return int(self._lib.vl1_batch_kernel_launches(self.handle))

    def eval(self, stream=None):
        import torch

        sh = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(self._lib.vl1_batch_eval(self.handle, C.c_void_p(sh)), "vl1_batch_eval")

    def capture(self):
        """Record one evaluation in a CUDA graph (after one plain run)."""
        import torch

        self.eval()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.eval(torch.cuda.current_stream().cuda_stream)
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            raise RuntimeError("capture() the batch first")
        self.graph.replay()

    def raise_on_status(self):
        import torch

        sh = torch.cuda.current_stream().cuda_stream
        seen = set()
        for p in self.problems:
            if id(p.plan) not in seen:
                seen.add(id(p.plan))
                p.plan.raise_on_status(sh)

    def close(self):
        if getattr(self, "handle", None):
            self.graph = None
            self._lib.vl1_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _time_batch(batch, reps):
    import torch

    batch.eval()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ts = []
    for _ in range(reps):
        ev[0].record()
        batch.eval()
        ev[1].record()
        ev[1].synchronize()
        ts.append(ev[0].elapsed_time(ev[1]))
    return float(np.median(ts))


_tuned: dict = {}


def _signature(problems):
    return tuple((int(p.view.n_target_boxes), int(p.keep["lists"].numel()), p.nrhs,
                  int(p.plan.nq), id(p.plan)) for p in problems)


def _plan_label(plan):
    return f"{plan.dim}d_q{plan.quad_order}" + ("_complex" if plan.complex_table else "")


def autotune_batch(problems, *, reps=3, divisors=(1, 2, 3, 4, 6, 8), shapes=True,
                   verbose=False):
    """Choose the tile shapes and the work-item size of a batch by timing.

    1. Tile shapes (when ``shapes``): for each plan of the batch in turn (the
       others at their best so far), every shape it can take (K chunk of 16
       or 32 source points per pipeline unit, 16, 32 or 64 output columns per
       CTA; ``Plan.mixed_shapes``) is set and the batch built and timed; the
       fastest shape is kept.
    2. Work-item size: candidates cap the keys of one work item at the mean
       (tile key, column chunk) count per SM divided by each of ``divisors``
       (smaller items balance the persistent launch better, larger ones pay
       fewer start-ups).
    Every candidate batch is timed by the median of ``reps`` evaluations
    (CUDA events).  Returns the fastest batch and the timing table; choices
    are cached per problem-set signature.  (The reference's tuning point is
    its kernel choice, ``list1.py:1240-1258``.)
    """
    import torch

    sig = _signature(problems)
    plans = []
    for p in problems:
        if all(p.plan is not q for q in plans):
            plans.append(p.plan)
    if sig in _tuned:
        chosen, cap = _tuned[sig]
        for pl in plans:
            pl.set_mixed_geometry(*chosen[id(pl)])
        return MixedBatch(problems, max_keys_per_item=cap), {"cached": True}
    stream = torch.cuda.current_stream().cuda_stream
    n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    table = {"shapes": {}, "caps": {}}

    def timed(cap):
        t0 = time.perf_counter()
        b = MixedBatch(problems, max_keys_per_item=cap)
        ms = _time_batch(b, reps)
        return b, ms, time.perf_counter() - t0

    best_ms = None
    if shapes:
        for pl in plans:
            label = _plan_label(pl)
            geo = pl.mixed_geometry()
            current = (geo["kc"], geo["nch"])
            rows = {}
            best_shape = current
            for shape in pl.mixed_shapes():
                pl.set_mixed_geometry(*shape)
                b, ms, build_s = timed(None)
                b.close()
                rows[f"kc{shape[0]}_nch{shape[1]}"] = {"ms": ms, "build_s": build_s}
                if verbose:
                    print(f"autotune {label}: kc {shape[0]}, nch {shape[1]} -> {ms:.3f} ms")
                if best_ms is None or ms < best_ms:
                    best_ms, best_shape = ms, shape
            pl.set_mixed_geometry(*best_shape)
            rows["chosen"] = f"kc{best_shape[0]}_nch{best_shape[1]}"
            table["shapes"][label] = rows
    total_keys = 0
    for p in problems:
        sch = get_schedule(p.plan, p.view, p.keep, p.nrhs, stream)
        geo = p.plan.mixed_geometry()
        total_keys += sch.n_tile_keys * (geo["np"] // geo["nch"])
    share = max(1, -(-total_keys // n_sm))
    best = None
    for d in (None,) + tuple(divisors):
        cap = None if d is None else max(2, -(-share // d))
        if str(cap) in table["caps"]:
            continue
        b, ms, build_s = timed(cap)
        table["caps"][str(cap)] = {"ms": ms, "build_s": build_s}
        if verbose:
            print(f"autotune: cap {cap} keys -> {ms:.3f} ms")
        if best is None or ms < best[0]:
            if best is not None:
                best[2].close()
            best = (ms, cap, b)
        else:
            b.close()
    chosen = {}
    for pl in plans:
        geo = pl.mixed_geometry()
        chosen[id(pl)] = (geo["kc"], geo["nch"])
    _tuned[sig] = (chosen, best[1])
    table["chosen"] = {"shapes": {_plan_label(pl): f"kc{chosen[id(pl)][0]}_nch{chosen[id(pl)][1]}"
                                  for pl in plans},
                       "cap": best[1], "ms": best[0]}
    return best[2], table
