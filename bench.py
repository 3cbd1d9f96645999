#!/usr/bin/env python
"""Benchmark of the GB300 list-1 near-field evaluation.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c2|c1|c3]

Workload (default ``c2``): 3D Laplace volume potential, list-1 near field only,
FP64, adaptive 2:1-balanced octree on [-0.5, 0.5]^3 refined where the density
variation over a leaf exceeds 1e-3 (23,087 leaves, q=4, 1,477,568 points),
density a sum of 16 seeded Gaussians; the canonical 3D Laplace table built
by Duffy quadrature in FP64 (the package's GPU builder at the reference's
default orders, outside the timed region).

One step = one list-1 evaluation of all target points for one right-hand side
(the reference's ``near_field`` launch).  Between timed steps the L2 cache is
flushed by writing a 256 MiB buffer (outside the timed events).  ``value`` is
points/s with every input resident in HBM (CUDA events on the launching
stream); ``e2e`` is the same metric through the public API
(``NearFieldFromCSR.__call__``) with the density copied from pinned host
memory and the potential copied back every step.

``--impl reference`` times the reference algorithm on the host cores: the C
restatement of ``volumential/list1.py``'s ``near_field`` kernel (the pocl CPU
path of the reference cannot run without pyopencl/loopy), one OpenMP work item
per target box, on a bounded sample of the same workload per step.

With N > 1 (torchrun) every rank runs an independent replica of the workload
(the path has no exchange step); ranks synchronise with a barrier around the
timed region and the maximum time over ranks is reported.
"""

from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "list-1 near-field pts/s & solves/s at ≤1e-9 rel err vs FP64; p50/p99 latency"
L2_FLUSH_BYTES = 256 << 20


def parse_args(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[1])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    p.add_argument("--workload", choices=("c2", "c1", "c3", "c4", "c5", "table", "csr",
                                          "split", "tree"),
                   default="c2")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--c4-problems", type=int, default=64, help="C4: problems in the batch")
    p.add_argument("--c4-max-level", type=int, default=6, help="C4: deepest uniform level")
    p.add_argument("--c5-requests", type=int, default=10000, help="C5: requests per run")
    p.add_argument("--c5-budget-gb", type=float, default=64.0,
                   help="C5: HBM budget of the resident plans, trees and schedules")
    p.add_argument("--c5-step", type=int, default=256, help="C5: most requests per step")
    p.add_argument("--c5-new", type=int, default=12,
                   help="C5: Helmholtz problems (continuous k) arriving with tables to build")
    p.add_argument("--c5-pressure", type=float, default=0.5,
                   help="C5 arrivals leg: HBM budget as a fraction of the mix's resident set")
    p.add_argument("--c5-build-ctas", type=int, default=-1,
                   help="C5 arrivals leg: CTAs of a table build (0: one per work item, "
                        "-1: a quarter of the SMs)")
    p.add_argument("--c5-rates", default="0.25,0.5,0.75,0.9",
                   help="C5: open-loop arrival rates as fractions of the closed-loop rate")
    p.add_argument("--cpu-seconds", type=float, default=10.0,
                   help="target CPU time of the cpu_baseline sample")
    return p.parse_args(argv)


# {{{ environment

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value):
    """The largest ``value`` over the ranks of the default process group (the
    value itself without one): replicas report the slowest rank's time."""
    import torch

    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, world, total_ms):
    """Whole-job throughput of ``world`` replicas that each processed
    ``units_per_rank`` units, timed by the slowest rank (``total_ms``)."""
    return world * units_per_rank / (total_ms / 1e3)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d.get("bf16_tflops", 1900.0)), "measured"
    return 6800.0, 1900.0, "fallback"


def measured_fp64_gflops(n=4096, reps=5):
    """FP64 peak of this GPU as cuBLAS DGEMM reaches it (2 n^3 flops per
    call, best of ``reps``, CUDA events): the denominator of the FP64-pipe
    roofline of the plain kernel, measured in the same run."""
    import torch

    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    c = a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b, c
    return 2.0 * n ** 3 / best / 1e9


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            for name, val in zip(names, r[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}

# }}}


def build_workload(name):
    from volumential_gb300 import workloads as W
    if name == "c1":
        return W.config_c1()
    if name == "c3":
        return W.config_c3()
    return W.config_c2()


def algorithmic_bytes(w, nrhs=1, out_complex=False, coef_complex=False, table_bytes=8):
    """Compulsory bytes of one list-1 evaluation (each array touched once)."""
    tr = w.traversal
    n = w.n_points
    ntb = len(tr.target_boxes)
    s_in = 16 if coef_complex else 8
    s_out = 16 if out_complex else 8
    n_compact = sum(int(np.asarray(t.get_reduced_table_data()[1]).size) for t in w.tables)
    return (n * nrhs * (s_in + s_out) + 4 * (ntb + 1) + 4 * tr.nnz + 4 * ntb
            + w.tree.nboxes * (8 * w.dim + 1 + 4 + 4) + n_compact * table_bytes + 2048)


def _timed_steps(torch, fn, flush, steps, stream, lib=None):
    """Run ``fn`` ``steps`` times, each bracketed by CUDA events on ``stream``
    with an L2 flush before it (outside the events); returns per-step ms and,
    with ``lib``, the per-step ms of the tensor-core kernel alone (events the
    library records around that launch, ``vl1_set_kernel_events``)."""
    import ctypes as C

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    kev = None
    if lib is not None:
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for a, b in kev:          # create the events' handles
            a.record(stream)
            b.record(stream)
        torch.cuda.synchronize()
    for i, (e0, e1) in enumerate(evs):
        flush.fill_(1.0)
        if kev:
            lib.vl1_set_kernel_events(C.c_void_p(kev[i][0].cuda_event),
                                      C.c_void_p(kev[i][1].cuda_event))
        e0.record(stream)
        fn()
        e1.record(stream)
    if kev:
        lib.vl1_set_kernel_events(None, None)
    torch.cuda.synchronize()
    ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    return ms, ([a.elapsed_time(b) for a, b in kev] if kev else None)


def gpu_arm(args):
    import torch

    from volumential_gb300.batched import eval_mixed, get_schedule
    from volumential_gb300.expansion_wrangler_fpnd import (
        FPNDExpansionWrangler,
        FPNDTreeIndependentDataForWrangler,
    )
    from volumential_gb300.plan import as_device_tensor, tree_view_from_arrays

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    w = build_workload(args.workload)
    ti = FPNDTreeIndependentDataForWrangler(target_kernels=[w.kernel])
    dtype = np.complex128 if w.kernel.is_complex_valued else np.float64
    wr = FPNDExpansionWrangler(ti, w.traversal, w.tables, dtype=dtype, quad_order=w.q)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, None)
    # resident tree arrays (device tensors) for both the kernel and the API runs
    tree_keys = ("target_boxes", "neighbor_source_boxes_starts",
                 "neighbor_source_boxes_lists", "box_centers", "box_levels",
                 "box_source_starts", "box_source_counts_nonchild", "box_target_starts",
                 "box_target_counts_nonchild", "source_mode_ids", "target_point_ids")
    for k in tree_keys:
        kw[k] = as_device_tensor(kw[k])
    plan = nf.get_plan(
        table_data_combined=kw["table_data_combined"],
        mode_nmlz_combined=kw["mode_nmlz_combined"], case_indices=kw["case_indices"],
        encoding_base=kw["encoding_base"], encoding_shift=kw["encoding_shift"],
        table_root_extent=kw["table_root_extent"],
        table_starting_level=kw["table_starting_level"],
        **{n: kw[n] for n in kw if n.startswith("arithmetic_")})
    view, keep = tree_view_from_arrays(root_extent=kw["root_extent"],
                                       **{k: kw[k] for k in tree_keys})
    n = w.n_points
    nrhs = w.nrhs
    coef_np = np.ascontiguousarray(w.coefs.reshape(nrhs, n))
    coef_complex = np.iscomplexobj(coef_np)
    coefs = as_device_tensor(coef_np).reshape(-1)
    out_complex = plan.complex_table or coef_complex
    odt = torch.complex128 if out_complex else torch.float64
    out_plain = torch.empty(nrhs * n, dtype=odt, device="cuda")
    out_mixed = torch.empty(nrhs * n, dtype=odt, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    def plain_step():
        plan.eval_fp64(view, coefs, out_plain, stream=sh, nrhs=nrhs)

    def mixed_step():
        eval_mixed(plan, view, coefs, out_mixed, stream=sh, nrhs=nrhs, keep=keep)

    # the steady-state schedule of a tree evaluated many times: host greedy
    # tile packing (the public API's first call on a new tree builds its
    # schedule on the device instead; e2e_cold below)
    t_sched = time.perf_counter()
    sched = get_schedule(plan, view, keep, nrhs, sh, packing="greedy")
    t_sched = time.perf_counter() - t_sched
    for _ in range(args.warmup):
        flush.fill_(1.0)
        plain_step()
        mixed_step()
    plan.raise_on_status(sh)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    res = {}
    from volumential_gb300 import _lib
    for name, fn in (("plain", plain_step), ("mixed", mixed_step)):
        step_ms, kernel_ms = _timed_steps(torch, fn, flush, args.steps, stream,
                                          _lib.lib() if name == "mixed" else None)
        total = max_over_ranks(float(sum(step_ms)))
        res[name] = {"step_ms": step_ms, "total_ms": total, "kernel_ms": kernel_ms}
    if world > 1:
        torch.distributed.barrier()
    clock_info = clocks.stop()
    plan.raise_on_status(sh)
    yp = out_plain.cpu().numpy().reshape(nrhs, n)
    ym = out_mixed.cpu().numpy().reshape(nrhs, n)
    mixed_errs = [float(np.linalg.norm(ym[r] - yp[r]) / np.linalg.norm(yp[r]))
                  for r in range(nrhs)]
    mixed_err = max(mixed_errs)
    headline = "plain"
    if mixed_err <= 1e-9 and res["mixed"]["total_ms"] < res["plain"]["total_ms"]:
        headline = "mixed"   # the faster path within its tolerance

    # e2e through the public API: pinned host densities in, host potentials
    # out (one rhs: NearFieldFromCSR.__call__; many: the wrangler's batched
    # eval_direct_batched)
    host_in = torch.from_numpy(coef_np if nrhs > 1 else coef_np[0]).pin_memory()
    host_out = torch.empty((nrhs, n) if nrhs > 1 else (n,), dtype=odt).pin_memory()
    dev_in = torch.empty(n, dtype=coefs.dtype, device="cuda")
    dev_out = torch.empty(n, dtype=odt, device="cuda")
    api_kw = dict(kw)
    api_kw.pop("mode_coefs", None)
    precision = "mixed" if headline == "mixed" else "fp64"
    nf.extra_kwargs["list1_precision"] = precision

    def api_step():
        if nrhs > 1:
            r_ = wr.eval_direct_batched(tr.target_boxes, tr.neighbor_source_boxes_starts,
                                        tr.neighbor_source_boxes_lists, host_in,
                                        precision=precision)[0][0]
        else:
            dev_in.copy_(host_in, non_blocking=True)
            r_, _ = nf(None, result=dev_out, mode_coefs=dev_in, **api_kw)
        host_out.copy_(r_, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    for _ in range(max(1, args.warmup)):
        api_step()
    e2e_ms = []
    gc.collect()
    gc.disable()        # no collector pauses inside the host-timed steps
    try:
        for _ in range(args.steps):
            flush.fill_(2.0)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            api_step()
            e2e_ms.append((time.perf_counter() - t1) * 1e3)
    finally:
        gc.enable()
    e2e_total = max_over_ranks(float(sum(e2e_ms)))
    api_err = float(np.linalg.norm(host_out.numpy().reshape(nrhs, n) - yp) / np.linalg.norm(yp))

    # e2e_cold: the same public call on a tree the library has not seen (new
    # device arrays every step): tree validation, the schedule built on the
    # device and its work items run inside the timed region; the caller's
    # copy of its tree arrays does not (one rhs: NearFieldFromCSR.__call__)
    cold = None
    if nrhs == 1:
        cold_ms = []
        n_cold = max(3, min(args.steps, 10))
        for i in range(n_cold + 1):
            fresh = {k: kw[k].clone() for k in tree_keys}
            cold_kw = dict(api_kw, **fresh)
            flush.fill_(3.0)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            dev_in.copy_(host_in, non_blocking=True)
            r_, _ = nf(None, result=dev_out, mode_coefs=dev_in, **cold_kw)
            host_out.copy_(r_, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            if i > 0:   # the first cold call also loads the builder's kernels
                cold_ms.append((time.perf_counter() - t1) * 1e3)
            del fresh, cold_kw
        cold = {"ms": cold_ms,
                "err": float(np.linalg.norm(host_out.numpy().reshape(nrhs, n) - yp) /
                             np.linalg.norm(yp))}

    return {
        "w": w, "res": res, "clocks": clock_info, "e2e_total_ms": e2e_total,
        "e2e_ms": e2e_ms, "out": yp[0], "out_complex": out_complex, "nrhs": nrhs,
        "coef_complex": coef_complex, "h2d": int(host_in.numel() * host_in.element_size()),
        "d2h": int(host_out.numel() * host_out.element_size()),
        "plan_bytes": plan.device_bytes(), "world": world, "rank": rank,
        "mixed_err": mixed_err, "mixed_errs": mixed_errs, "api_err": api_err, "cold": cold,
        "headline": headline, "fp64_gflops": measured_fp64_gflops(),
        "schedule": {"tiles": sched.n_tiles, "tile_keys": sched.n_tile_keys,
                     "mean_keys_per_tile": sched.mean_keys_per_tile,
                     "build_s": t_sched, "workspace_bytes": int(sched.workspace_bytes)},
        "geometry": plan.mixed_geometry(),
    }


def oracle_sample(w, fraction, nthreads=0, seed=0):
    """Time the C oracle on a seeded sample of target boxes; returns
    (seconds, sampled points, sampled target point ids, result values)."""
    from tests.helpers import oracle_for_workload  # test infrastructure
    from tests.helpers import LAP2, LAP3, FIXED
    policy = {"c1": LAP2, "c2": LAP3, "c3": FIXED}
    tr = w.traversal
    ntb = len(tr.target_boxes)
    rng = np.random.default_rng(seed)
    k = max(1, int(round(fraction * ntb)))
    pick = np.sort(rng.choice(ntb, size=k, replace=False))
    st = tr.neighbor_source_boxes_starts
    lens = st[pick + 1] - st[pick]
    sub_starts = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    sub_lists = np.concatenate([tr.neighbor_source_boxes_lists[st[i]:st[i + 1]]
                                for i in pick]).astype(np.int32)
    tree = w.tree
    name = "c2" if w.dim == 3 else ("c3" if w.kernel.is_complex_valued else "c1")
    prob = oracle_for_workload(w, policy[name])
    local = tree.box_local_mode_ids()
    t0 = time.perf_counter()
    res = prob.near_field(
        target_boxes=tr.target_boxes[pick], neighbor_source_boxes_starts=sub_starts,
        neighbor_source_boxes_lists=sub_lists, box_centers=tree.box_centers,
        box_levels=tree.box_levels, box_source_starts=tree.box_target_starts,
        box_source_counts_nonchild=tree.box_target_counts_nonchild,
        box_target_starts=tree.box_target_starts,
        box_target_counts_nonchild=tree.box_target_counts_nonchild,
        source_mode_ids=local, target_point_ids=local, mode_coefs=w.coefs[0],
        nthreads=nthreads)
    dt = time.perf_counter() - t0
    nq = w.q ** w.dim
    ids = (tree.box_target_starts[tr.target_boxes[pick]][:, None]
           + np.arange(nq)[None, :]).ravel()
    return dt, int(k * nq), ids, res[ids]


def calibrated_fraction(w, seconds, nthreads):
    frac = 0.002
    while True:
        dt, _, _, _ = oracle_sample(w, frac, nthreads)
        if dt > 0.5 or frac >= 1.0:
            break
        frac = min(1.0, frac * 4)
    return min(1.0, frac * seconds / max(dt, 1e-3))


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    w = build_workload(args.workload)
    nthreads = os.cpu_count() or 1
    budget = min(10.0, 150.0 / max(1, args.warmup + args.steps))
    frac = calibrated_fraction(w, budget, nthreads)
    for i in range(args.warmup):
        oracle_sample(w, frac, nthreads, seed=i)
    times, pts = [], 0
    for i in range(args.steps):
        dt, n, _, _ = oracle_sample(w, frac, nthreads, seed=1000 + i)
        times.append(dt)
        pts += n
    total = sum(times)
    value = pts / total
    sample = (f"{frac * 100:.2f}% of the target boxes per step (seeded), "
              f"{pts // args.steps} target points per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "points/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(w),
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": nthreads,
                         "kind": "port", "sample": f"{sample}, {cpu_model()}",
                         "nrhs_timed": 1},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)
    return 0


def _cold_summary(r, n, nrhs):
    """e2e_cold of the JSON line: points/s of first calls on new trees."""
    c = r.get("cold")
    if not c:
        return None
    ms = np.asarray(c["ms"])
    warm = float(np.mean(r["e2e_ms"]))
    return {"value": n * nrhs / (float(np.mean(ms)) / 1e3), "unit": "points/s",
            "latency_ms": {"p50": float(np.percentile(ms, 50)),
                           "p99": float(np.percentile(ms, 99))},
            "ratio_to_warm_e2e": float(np.mean(ms)) / warm, "steps": int(ms.size),
            "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"],
            "rel_l2_vs_fp64": c["err"], "schedule": "built on the device per call",
            "api": "NearFieldFromCSR.__call__ on new device tree arrays each step"}


def workload_config(w):
    """The workload's description, shared by both arms' JSON lines."""
    return {"workload": w.name, "dim": w.dim, "q": w.q, "nrhs": w.nrhs,
            "points": w.n_points, "leaves": int(len(w.traversal.target_boxes)),
            "list1_box_pairs": w.traversal.nnz, "point_pairs": w.pair_count(),
            "tables": _table_source(w)}


def _per_rhs(errs):
    """Relative l2 error of every right-hand side (rounded) and its spread."""
    e = np.asarray(errs, dtype=np.float64)
    return {"n": int(e.size), "min": float(e.min()), "median": float(np.median(e)),
            "max": float(e.max()), "values": [float(f"{x:.3g}") for x in e]}


def _table_source(w):
    if w.meta.get("tables") == "duffy":
        t = w.tables[0]
        return (f"FP64 Duffy quadrature on the GPU ({type(t.integral_knl).__name__}, "
                f"q={t.quad_order}, source box extent {t.source_box_extent:g}, regular 20 / "
                "radial 61 tanh-sinh-fast)")
    return "seeded synthetic values in the compact layout"


def tensor_executed(r, ms_per_step, bf16_peak):
    g = r["geometry"]
    flops = 2.0 * 15 * 128 * r["schedule"]["tile_keys"] * g["kp"] * g["np"]
    tflops = flops / (ms_per_step / 1e3) / 1e12
    return {"flops_per_step": flops, "tflops": tflops, "frac_of_bf16_peak": tflops / bf16_peak,
            "note": "FP16 digit-pair MMAs (M=128 rows x N=np x K=kp) per tile key"}


def gb300_main(args):
    world, rank, _ = dist_env()
    r = gpu_arm(args)
    w = r["w"]
    K = args.steps
    n = w.n_points
    nrhs = r["nrhs"]
    hbm, bf16, peak_kind = peaks()
    B = algorithmic_bytes(w, nrhs=nrhs, out_complex=r["out_complex"],
                          coef_complex=r["coef_complex"],
                          table_bytes=16 if w.tables[0].dtype == np.complex128 else 8)
    P = w.pair_count()
    # FP64-equivalent algorithmic flops: 2 per point pair and rhs, 4 for a
    # complex table (digit slices of the tensor-core path not counted)
    F = (4 if r["out_complex"] else 2) * P * nrhs
    fp64_peak = r["fp64_gflops"]

    def path_summary(name):
        step_ms = np.asarray(r["res"][name]["step_ms"])
        t = float(np.mean(step_ms)) / 1e3
        return {
            "value": replica_rate(n * nrhs * K, world, r["res"][name]["total_ms"]),
            "ms_per_step": r["res"][name]["total_ms"] / K,
            "latency_ms": {"p50": float(np.percentile(step_ms, 50)),
                           "p99": float(np.percentile(step_ms, 99))},
            "hbm_gbs": B / t / 1e9, "hbm_frac": B / t / 1e9 / hbm,
            "fp64eq_tflops": F / t / 1e12,
        }

    plain = path_summary("plain")
    mixed = path_summary("mixed")
    plain.update({"fp64_gflops": F / (plain["ms_per_step"] / 1e3) / 1e9,
                  "fp64_peak_gflops_measured_dgemm": fp64_peak,
                  "fp64_frac_of_measured_dgemm":
                      F / (plain["ms_per_step"] / 1e3) / 1e9 / fp64_peak})
    head = mixed if r["headline"] == "mixed" else plain
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(f"{r['headline']}/{w.name}")
    kms = r["res"]["mixed"]["kernel_ms"]
    if r["headline"] == "mixed" and kms:
        # the dominant kernel (mixed_kernel) timed alone with events the
        # library records around its launch, inside the timed steps.
        # T_roof = max(B / HBM, F / tensor peak), F the FP64-equivalent
        # algorithmic flops; frac = T_roof / T_kernel
        kernel_s = float(np.mean(kms)) / 1e3
        t_hbm, t_pipe = B / (hbm * 1e9), F / (bf16 * 1e12)
        if t_pipe >= t_hbm:
            roof = {"bound": "tensor", "achieved": F / kernel_s / 1e12, "peak": bf16,
                    "unit": "TFLOP/s"}
        else:
            roof = {"bound": "hbm", "achieved": B / kernel_s / 1e9, "peak": hbm,
                    "unit": "GB/s"}
        roof.update({"frac": max(t_hbm, t_pipe) / kernel_s, "kernel": "mixed_kernel",
                     "kernel_ms": kernel_s * 1e3,
                     "kernel_share_of_step": kernel_s * 1e3 / head["ms_per_step"]})
    else:
        # the FP64 kernel: its binding roof is the FP64 pipe (2 flops per point
        # pair per rhs), against the DGEMM rate measured in this run
        kernel_s = head["ms_per_step"] / 1e3
        t_hbm, t_pipe = B / (hbm * 1e9), F / (fp64_peak * 1e9)
        roof = {"bound": "fp64", "achieved": F / kernel_s / 1e9, "peak": fp64_peak,
                "unit": "GFLOP/s", "frac": max(t_hbm, t_pipe) / kernel_s,
                "kernel": "plain_kernel", "peak_note": "cuBLAS DGEMM measured in this run"}
    roof.update({"traffic": traffic,
                 "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu "
                                   "capture of this kernel on this workload "
                                   "(profiles/traffic.json), not measured in this run",
                 "peak_source": peak_kind, "algorithmic_bytes": int(B),
                 "algorithmic_flops_fp64eq": int(F),
                 "roof_time_us": 1e6 * max(t_hbm, t_pipe)})

    line = {
        "metric": METRIC, "value": head["value"], "unit": "points/s", "n_gpus": world,
        "steps": K, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16-digits/fp32-exact/f64" if r["headline"] == "mixed" else "f64",
        "data": "synthetic",
        "config": workload_config(w),
        "path": r["headline"], "l2": "flushed between steps (256 MiB write)",
        "parallelism": "replicas" if world > 1 else "single",
        "rel_l2_vs_fp64": r["mixed_err"] if r["headline"] == "mixed" else 0.0,
        "rel_l2_per_rhs": _per_rhs(r["mixed_errs"]) if r["headline"] == "mixed" else None,
        "solves_per_s": 1e3 * nrhs / head["ms_per_step"],
        "latency_ms": head["latency_ms"],
        "e2e": {"value": replica_rate(n * nrhs * K, world, r["e2e_total_ms"]), "unit": "points/s",
                "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"],
                "latency_ms": {"p50": float(np.percentile(r["e2e_ms"], 50)),
                               "p99": float(np.percentile(r["e2e_ms"], 99))},
                "rel_l2_vs_fp64": r["api_err"],
                "api": "NearFieldFromCSR.__call__" if nrhs == 1
                       else "FPNDExpansionWrangler.eval_direct_batched"},
        "e2e_cold": _cold_summary(r, n, nrhs),
        "roofline": roof,
        "paths": {"plain_fp64": plain, "mixed": dict(mixed, rel_l2_vs_fp64=r["mixed_err"]),
                  "speedup_mixed_over_plain": plain["ms_per_step"] / mixed["ms_per_step"]},
        "mixed_schedule": r["schedule"], "mixed_geometry": r["geometry"],
        # digit products the tensor pipe executes per step (15 FP16 digit
        # pairs per source/target point pair of every tile row, padding
        # included), next to the FP64-equivalent algorithmic flops above
        "tensor_executed": tensor_executed(r, mixed["ms_per_step"], bf16),
        "clocks": r["clocks"],
        "gpu_launches": K * (1 if r["headline"] == "plain" else (3 if w.dim == 3 else 5)),
        "plan_device_bytes": r["plan_bytes"],
    }

    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        nthreads = os.cpu_count() or 1
        frac = calibrated_fraction(w, args.cpu_seconds, nthreads)
        dt, pts, ids, ref = oracle_sample(w, frac, nthreads, seed=7)
        got = r["out"][ids]
        err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        line["cpu_baseline"] = {
            "value": pts / dt, "unit": "points/s", "cores": nthreads, "kind": "port",
            "sample": f"{frac * 100:.2f}% of the target boxes (seeded), {pts} target points, "
                      f"{dt:.1f} s on {cpu_model()}"}
        line["rel_l2_plain_vs_oracle_sample"] = err
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def c4_main(args):
    """Uneven batch (C4): 64 uniform 3D Laplace problems of levels 3..6,
    q in {3, 4, 5}, 1..32 right-hand sides each (FP64 Duffy tables per q),
    evaluated by one CUDA-graph-captured batch (batched preparation + one
    persistent tensor-core launch per kernel shape, problems that fill the GPU
    alone with their own launch) whose tile shapes and work-item size are
    autotuned.  One step = one replay of the graph over all problems;
    compared with the same problems evaluated one by one (mixed path, same
    schedules) and with the FP64 kernel (one pass each), and the errors of
    every (problem, rhs) against the FP64 results."""
    import ctypes as C

    import torch

    from volumential_gb300 import _lib
    from volumential_gb300 import workloads as W
    from volumential_gb300.batch import BatchProblem, autotune_batch, plan_for, tree_arrays

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    ws = W.config_c4(n_problems=args.c4_problems, levels=(3, args.c4_max_level))
    t_host = time.perf_counter() - t0
    t0 = time.perf_counter()
    plans, views, probs = {}, {}, []
    for w in ws:
        if w.meta["table_key"] not in plans:
            plans[w.meta["table_key"]] = plan_for(w)
        if w.meta["tree_key"] not in views:      # one copy of a tree on the device
            views[w.meta["tree_key"]] = tree_arrays(w)
        view, keep = views[w.meta["tree_key"]]
        pts = torch.from_numpy(np.ascontiguousarray(w.tree.targets)).to("cuda")
        coefs = torch.empty((w.nrhs, w.n_points), dtype=torch.float64, device="cuda")
        for r, m in enumerate(w.meta["mixtures"]):
            coefs[r] = m.on_device(pts)
        del pts
        probs.append(BatchProblem(plans[w.meta["table_key"]], view, keep, coefs,
                                  torch.zeros_like(coefs), w.nrhs))
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch, table = autotune_batch(probs, reps=2)
    t_tune = time.perf_counter() - t0
    batch.capture()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        batch.replay()
    batch.raise_on_status()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    step_ms = []
    for _ in range(args.steps):
        ev[0].record(stream)
        batch.replay()
        ev[1].record(stream)
        ev[1].synchronize()
        step_ms.append(ev[0].elapsed_time(ev[1]))
    clock_info = clocks.stop()
    batch.raise_on_status()
    mem_peak = torch.cuda.max_memory_allocated()
    # comparisons, one problem at a time into one shared scratch output and
    # one shared workspace: (a) each problem alone through vl1_eval_mixed with
    # the batch's schedule (bit-identical to the batch), (b) the FP64 kernel
    sh = stream.cuda_stream
    lib = _lib.lib()
    tmp = torch.empty(max(p.out.numel() for p in probs), dtype=torch.float64, device="cuda")
    wsp = torch.empty(max(sc.workspace_bytes for sc in batch.schedules), dtype=torch.uint8,
                      device="cuda")

    def separate(p, sc):
        _lib.check(lib.vl1_eval_mixed(p.plan.handle, C.byref(p.view), C.byref(sc.c_struct),
                                      p.coefs.data_ptr(), p.nrhs, tmp.data_ptr(),
                                      wsp.data_ptr(), wsp.numel(), C.c_void_p(sh)),
                   "vl1_eval_mixed")

    for p, sc in zip(probs, batch.schedules):   # untimed pass (kernel loading)
        separate(p, sc)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for p, sc in zip(probs, batch.schedules):
        separate(p, sc)
    ev[1].record(stream)
    ev[1].synchronize()
    sep_ms = ev[0].elapsed_time(ev[1])
    same = True
    for p, sc in zip(probs, batch.schedules):
        separate(p, sc)
        same = same and torch.equal(tmp[:p.out.numel()].view_as(p.out), p.out)
    plain_ms, errs = 0.0, []
    for p in probs:
        ev[0].record(stream)
        p.plan.eval_fp64(p.view, p.coefs, tmp[:p.out.numel()], stream=sh, nrhs=p.nrhs)
        ev[1].record(stream)
        ev[1].synchronize()
        plain_ms += ev[0].elapsed_time(ev[1])
        ref = tmp[:p.out.numel()].view(p.nrhs, -1)
        d = (p.out.view(p.nrhs, -1) - ref)
        errs.extend((torch.linalg.norm(d, dim=1) / torch.linalg.norm(ref, dim=1)).tolist())
    pts = sum(int(p.view.n_particles) * p.nrhs for p in probs)
    pairs = sum(w.pair_count() * w.nrhs for w in ws)
    ms = float(np.mean(step_ms))
    hbm, bf16, peak_kind = peaks()
    levels = [w.meta["level"] for w in ws]
    line = {
        "metric": METRIC, "value": pts / (ms / 1e3), "unit": "points/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16-digits/fp32-exact/f64", "data": "synthetic",
        "config": {"workload": f"c4_lap3d_uniform_batch{len(probs)}", "problems": len(probs),
                   "levels": [3, args.c4_max_level],
                   "problems_per_level": {str(l): levels.count(l)
                                          for l in range(3, args.c4_max_level + 1)},
                   "q": [3, 4, 5], "nrhs": [1, 32], "points_x_rhs": pts,
                   "point_pairs_x_rhs": pairs,
                   "tables": "; ".join(sorted({_table_source(w) for w in ws})),
                   "l2": "inputs (%.1f GB) far larger than L2" %
                         (sum(p.coefs.numel() * 8 for p in probs) / 1e9),
                   "path": "batch, CUDA graph replay", "waves": 1},
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)),
                       "p99": float(np.percentile(step_ms, 99))},
        "rel_l2_vs_fp64": {"max": max(errs), "median": float(np.median(errs)),
                           "n": len(errs)},
        "batch_equals_separate_mixed": bool(same),
        "paths": {"batch_graph_ms": ms, "separate_mixed_ms": sep_ms, "plain_fp64_ms": plain_ms,
                  "speedup_batch_over_plain": plain_ms / ms,
                  "speedup_batch_over_separate": sep_ms / ms},
        "autotune": table,
        "batch_device_bytes": batch.device_bytes, "device_bytes_peak": int(mem_peak),
        "setup_s": {"host_trees_tables": t_host, "device_inputs": t_setup},
        "autotune_s": t_tune, "pair_rate_per_s": pairs / (ms / 1e3),
        "e2e": None, "e2e_note": "resident-data batch; host copies of the inputs are not "
                                 "part of this configuration",
        "clocks": clock_info, "peak_source": peak_kind,
        "gpu_launches": args.steps * batch.kernel_launches,
    }
    if rank == 0:
        print(json.dumps(line, default=str), flush=True)
    return 0


def c5_main(args):
    """Serving (C5): ``--c5-requests`` single-rhs requests over a seeded mix of
    2D/3D Laplace and Helmholtz (k in 1..30) problems on uniform trees of
    1k..500k points (q in {3,4,5}), resident under an HBM budget and served by
    continuous batching (``volumential_gb300.serving``).  One step = one
    closed-loop run of all requests (submitted at once, steps of up to
    ``--c5-step`` requests, two in flight); then open-loop runs with Poisson
    arrivals at fractions of the closed-loop rate give p50/p99 latency, and
    the same requests one per step give the unbatched comparison."""
    import torch

    from volumential_gb300 import workloads as W
    from volumential_gb300.serving import ServingEngine, latency_stats

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    probs, reqs, mixes = W.config_c5(n_requests=args.c5_requests)
    ws = W.c5_workloads(probs)
    t_host = time.perf_counter() - t0
    eng = ServingEngine(hbm_budget_bytes=int(args.c5_budget_gb * (1 << 30)),
                        step_capacity_bytes=4 << 30, max_step_requests=args.c5_step)
    for key, w in ws.items():
        eng.register(key, w, w.meta["table_key"], w.meta["tree_key"], w.meta["sched_key"])
    t0 = time.perf_counter()
    dens, outs = {}, {}
    for key, w in ws.items():
        eng.admit(key)
        pts = torch.from_numpy(np.ascontiguousarray(w.tree.targets)).to("cuda")
        dens[key] = [m.on_device(pts).contiguous() for m in mixes[key]]
        outs[key] = torch.empty(w.n_points, dtype=torch.complex128
                                if w.kernel.is_complex_valued else torch.float64,
                                device="cuda")
    torch.cuda.synchronize()
    t_resident = time.perf_counter() - t0
    n_points = sum(probs[k].n_points for k, _ in reqs)

    def closed_loop():
        for key, di in reqs:
            eng.submit(key, dens[key][di], out=outs[key])
        ta = time.perf_counter()
        eng.drain()
        torch.cuda.synchronize()
        return time.perf_counter() - ta

    for _ in range(args.warmup):
        closed_loop()
    eng.check_status()
    clocks = ClockSampler(local)
    clocks.start()
    steps_before = eng.n_steps
    host0, gpu0 = eng.host_s, eng.gpu_ms
    runs = [closed_loop() for _ in range(args.steps)]
    clock_info = clocks.stop()
    n_batches = (eng.n_steps - steps_before) / max(args.steps, 1)
    host_frac = (eng.host_s - host0) / sum(runs)
    gpu_frac = (eng.gpu_ms - gpu0) / 1e3 / sum(runs)
    t_run = float(np.median(runs))
    rate = len(reqs) / t_run
    # open loop: Poisson arrivals at fractions of the closed-loop rate
    sweep = {}
    for frac in [float(x) for x in args.c5_rates.split(",") if x]:
        arr = W.poisson_arrivals(len(reqs), frac * rate, seed=int(frac * 1000))
        done, wall = eng.run([(float(t), k, dens[k][di], outs[k])
                              for t, (k, di) in zip(arr, reqs)])
        st = latency_stats(done)
        st["offered_per_s"] = frac * rate
        st["achieved_per_s"] = len(done) / wall
        sweep[f"{frac:g}"] = st
    # unbatched: one request per step, waiting for each
    n_serial = min(len(reqs), 2000)
    eng.max_step_requests = 1
    ta = time.perf_counter()
    for key, di in reqs[:n_serial]:
        eng.submit(key, dens[key][di], out=outs[key])
        eng.drain()
    torch.cuda.synchronize()
    serial_rate = n_serial / (time.perf_counter() - ta)
    eng.max_step_requests = args.c5_step
    # accuracy (vs the FP64 path) and alone-vs-mix identity on a sample
    rng = np.random.default_rng(5)
    sample = [reqs[i] for i in rng.choice(len(reqs), size=min(48, len(reqs)), replace=False)]
    mix_reqs = [eng.submit(k, dens[k][di]) for k, di in sample]
    for key, di in reqs[:200]:
        eng.submit(key, dens[key][di], out=outs[key])
    eng.drain()
    errs, same = [], True
    sh = torch.cuda.current_stream().cuda_stream
    for q, (key, di) in zip(mix_reqs, sample):
        alone = eng.submit(key, dens[key][di])
        eng.drain()
        same = same and torch.equal(alone.out, q.out)
        plan, (view, keep), _ = eng.admit(key)
        ref = torch.empty_like(q.out)
        plan.eval_fp64(view, dens[key][di], ref, stream=sh, nrhs=1)
        torch.cuda.synchronize()
        errs.append(float(torch.linalg.norm(q.out - ref) / torch.linalg.norm(ref)))
    eng.check_status()
    resident_set = eng.budget.used
    evictions = eng.budget.evictions
    pressure = c5_arrivals_leg(args, eng, ws, probs, reqs, dens, rate, resident_set) \
        if args.c5_new > 0 else None
    hbm, bf16, peak_kind = peaks()
    kinds = {}
    for key, _ in reqs:
        kk = f"{key[0]}d_{key[1]}"
        kinds[kk] = kinds.get(kk, 0) + 1
    line = {
        "metric": METRIC, "value": n_points / t_run, "unit": "points/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_run * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16-digits/fp32-exact/f64", "data": "synthetic",
        "config": {"workload": f"c5_serving_{len(reqs)}req", "requests": len(reqs),
                   "problems": len(probs), "tables": len({p.table_key for p in probs.values()}),
                   "trees": len({w.meta["tree_key"] for w in ws.values()}),
                   "mix": kinds, "points_range": [1000, 500000], "q": [3, 4, 5],
                   "helmholtz_k": [1, 30], "max_step_requests": args.c5_step,
                   "l2": "resident densities %.1f GB, far larger than L2" %
                         (sum(d.numel() * 8 for v in dens.values() for d in v) / 1e9),
                   "path": "continuous batching (vl1_batch_update + vl1_batch_eval)"},
        "solves_per_s": rate, "steps_per_run": n_batches,
        "closed_loop_time_shares": {"host_step_assembly": host_frac,
                                    "gpu_steps": gpu_frac},
        "latency_ms": sweep.get("0.5", next(iter(sweep.values()), {})),
        "open_loop": sweep,
        "unbatched_solves_per_s": serial_rate,
        "speedup_over_unbatched": rate / serial_rate,
        "rel_l2_max_vs_fp64": max(errs), "same_alone_and_in_mix": bool(same),
        "resident_bytes": resident_set, "hbm_budget_bytes": eng.budget.budget,
        "evictions": evictions,
        "arrivals_under_pressure": pressure,
        "setup_s": {"host": t_host, "resident": t_resident},
        "e2e": None, "e2e_note": "resident trees, tables and densities (the serving "
                                 "configuration); results stay on the device",
        "clocks": clock_info, "peak_source": peak_kind,
        "gpu_launches": int(round(n_batches * 7)),
    }
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def c5_arrivals_leg(args, eng, ws, probs, reqs, dens, closed_rate, resident_set):
    """C5 under memory pressure, with table builds on arrival.  Engines whose
    HBM budget is ``--c5-pressure`` times the mix's resident set serve
    requests over the mix's problems with Zipf popularity (s = 1.1, a seeded
    ranking; the most popular problems that fit 80 % of the budget are
    admitted before the clock, every other one is admitted cold and the
    least recently used idle entries are evicted).  (1) Closed loop: all
    requests at once, giving the sustainable rate under pressure.  (2) Open
    loop on a fresh engine: Poisson arrivals at half that rate, into which
    ``--c5-new`` new Helmholtz problems (k uniform in [1, 30], real) arrive
    one after another; the first request of a new problem starts the FP64
    Duffy build of its table on the engine's build thread while the engine
    keeps serving the others.  Reports latency percentiles (all requests,
    those that waited for a table build, the others), evictions, admissions
    and builds, the new problems' error against the FP64 path, and that
    sampled results are the same bits alone and in the mix."""
    import torch

    from volumential_gb300 import workloads as W
    from volumential_gb300.serving import ServingEngine, latency_stats

    for _ in range(2):   # release the first engine's residents (trees after schedules)
        eng.budget.make_room(eng.budget.budget)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    budget = int(args.c5_pressure * resident_set)
    keys = sorted(ws)
    rng = np.random.default_rng(77)
    rank = rng.permutation(len(keys))
    pop = 1.0 / (1.0 + rank) ** 1.1
    pop /= pop.sum()
    n_base = len(reqs)
    stream = [(keys[i], int(rng.integers(4))) for i in rng.choice(len(keys), size=n_base, p=pop)]

    serve_stream = torch.cuda.Stream(priority=-1)   # ahead of the table builds

    def engine():
        e = ServingEngine(hbm_budget_bytes=budget, step_capacity_bytes=4 << 30,
                          max_step_requests=args.c5_step, stream=serve_stream)
        for key, w in ws.items():
            e.register(key, w, w.meta["table_key"], w.meta["tree_key"], w.meta["sched_key"])
        for i in np.argsort(rank):
            if e.budget.used > 0.8 * budget:
                break
            e.admit(keys[i])
        torch.cuda.synchronize()
        return e

    # (1) closed loop under pressure
    e1 = engine()
    t0 = time.perf_counter()
    for key, di in stream:
        e1.submit(key, dens[key][di])
    e1.drain()
    torch.cuda.synchronize()
    closed_s = time.perf_counter() - t0
    closed = {"solves_per_s": n_base / closed_s, "evictions": e1.budget.evictions,
              "cold_admissions": e1.cold_admissions}
    e1.budget.make_room(budget)
    e1.budget.make_room(budget)
    e1.close()
    del e1
    torch.cuda.empty_cache()

    # (2) open loop at half the pressure rate, new problems arriving
    new_probs = W.config_c5_arrivals(n_new=args.c5_new)
    # by default builds run on a quarter of the SMs, the rest stay with the solves
    build_ctas = args.c5_build_ctas
    if build_ctas < 0:
        build_ctas = max(1, torch.cuda.get_device_properties(0).multi_processor_count // 4)
    new_ws, builders = W.c5_arrival_workloads(new_probs, build_ctas=build_ctas)
    eng2 = engine()
    new_dens = {}
    for key, w in new_ws.items():
        eng2.register(key, w, w.meta["table_key"], w.meta["tree_key"], w.meta["sched_key"],
                      build_tables=builders[key])
        pts = torch.from_numpy(np.ascontiguousarray(w.tree.targets)).to("cuda")
        mixes = [W.random_gaussian_mixture(rng, w.dim, int(rng.integers(4, 17)), (0.01, 0.1))
                 for _ in range(4)]
        new_dens[key] = [m.on_device(pts).contiguous() for m in mixes]
    all_dens = dict(dens)
    all_dens.update(new_dens)
    rate = 0.5 * closed["solves_per_s"]
    t_base = W.poisson_arrivals(n_base, rate, seed=78)
    span = float(t_base[-1])
    events = [(float(t), k, di) for t, (k, di) in zip(t_base, stream)]
    # new problem i starts at (0.1 + 0.5 i / n_new) of the run, then 24
    # requests within a fifth of it
    per_new = 24
    for i, key in enumerate(sorted(new_ws)):
        t0 = span * (0.1 + 0.5 * i / max(len(new_ws), 1))
        ts = t0 + W.poisson_arrivals(per_new, per_new / (0.2 * span), seed=90 + i)
        ts[0] = t0
        events += [(float(t), key, int(j % 4)) for j, t in enumerate(ts)]
    events.sort(key=lambda e: e[0])
    sample_ids = set(rng.choice(len(events), size=min(40, len(events)), replace=False).tolist())
    sample_ids |= {j for j, e in enumerate(events) if e[1] in new_ws and e[2] == 0}
    arrivals, outs = [], {}
    for j, (t, key, di) in enumerate(events):
        w = ws.get(key) or new_ws[key]
        dt = torch.complex128 if w.kernel.is_complex_valued else torch.float64
        if j in sample_ids:
            out = torch.empty(w.n_points, dtype=dt, device="cuda")
        else:
            out = outs.get(key)
            if out is None:
                out = outs[key] = torch.empty(w.n_points, dtype=dt, device="cuda")
        arrivals.append((t, key, all_dens[key][di], out))
    torch.cuda.synchronize()
    done, wall = eng2.run(arrivals)
    eng2.check_status()
    waited = [q for q in done if q.waited_build]
    rest = [q for q in done if not q.waited_build]
    # sampled requests again, one at a time: identical bits; new problems
    # against the FP64 path
    same, errs = True, []
    sh = serve_stream.cuda_stream
    for j in sorted(sample_ids):
        q = done[j]
        alone = eng2.submit(q.key, q.coefs)
        eng2.drain()
        same = same and torch.equal(alone.out, q.out)
        if q.key in new_ws:
            plan, (view, keep), _ = eng2.admit(q.key)
            ref = torch.empty_like(q.out)
            plan.eval_fp64(view, q.coefs, ref, stream=sh, nrhs=1)
            torch.cuda.synchronize()
            errs.append(float(torch.linalg.norm(q.out - ref) / torch.linalg.norm(ref)))
    eng2.check_status()
    out = {
        "hbm_budget_bytes": budget, "mix_resident_set_bytes": resident_set,
        "popularity": "Zipf s = 1.1 over the mix's problems (seeded ranking); the most "
                      "popular that fit 80 % of the budget admitted before the clock",
        "closed_loop": closed,
        "requests": len(done), "new_problems": len(new_ws),
        "new_problem_k": sorted(float(k[2]) for k in new_ws),
        "new_problem_shapes": sorted(f"{k[0]}d_q{k[3]}_l{k[4]}" for k in new_ws),
        "tables_built_on_arrival": eng2.table_builds,
        "table_build_ctas": build_ctas,
        "table_build_s_total": eng2.table_build_s,
        "table_source": "FP64 Duffy quadrature on the GPU per new k (reference default "
                        "orders), on the engine's build thread and stream",
        "offered_per_s": rate, "achieved_per_s": len(done) / wall, "wall_s": wall,
        # the resident problems' requests alone: served over the arrivals'
        # span (the run's wall time ends with the last table build)
        "others_achieved_per_s": len(rest) / max(
            max(q.t_done for q in rest) - min(q.arrival for q in done), 1e-9) if rest else None,
        "latency_ms": latency_stats(done),
        "latency_ms_waited_for_table_build": latency_stats(waited),
        "latency_ms_others": latency_stats(rest),
        "evictions": eng2.budget.evictions, "cold_admissions": eng2.cold_admissions,
        "rel_l2_max_vs_fp64_new_problems": max(errs) if errs else None,
        "same_alone_and_in_mix": bool(same), "sampled": len(sample_ids),
    }
    eng2.close()
    return out


def table_main(args):
    """FP64 table builder (``vl1_duffy_table``): full orbit-invariant tables
    at the reference's default Duffy orders (regular 20, radial 61,
    tanh-sinh-fast).  One step = one full build of each table (3D Laplace
    q=4; 2D Helmholtz q=5, k=20); the CPU restatement is timed on a sample of
    entries at lower orders and reported per quadrature node."""
    import torch

    from oracle import duffy_oracle as DO   # CPU baseline only
    from volumential_gb300 import table_builder as TB
    from volumential_gb300.kernels import HelmholtzKernel, LaplaceKernel
    from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    reg, rad = TB.DEFAULT_ORDERS["regular_quad_order"], TB.DEFAULT_ORDERS["radial_quad_order"]
    n_rad = len(TB.tanh_sinh_fast_rule(rad)[0])
    cases = [("lap3d_q4", 3, 4, LaplaceKernel(3), np.float64, None),
             ("helm2d_q5_k20", 2, 5, HelmholtzKernel(2), np.complex128, 20.0)]
    out = {}
    stream = torch.cuda.current_stream()
    for name, dim, q, knl, dt, k in cases:
        t = NearFieldInteractionTable(q, dim=dim, sumpy_kernel=knl, dtype=dt)
        ids = t._get_invariant_entry_info()["entry_ids"]
        nodes_per_entry = (2 ** dim) * (6 if dim == 3 else 2) * reg ** (dim - 1) * n_rad
        for _ in range(args.warmup):
            TB.build_table_values(t, entry_ids=ids[:256], k=k, store=False)
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            w0 = time.perf_counter()
            e0.record(stream)
            TB.build_table_values(t, k=k, store=False)
            e1.record(stream)
            e1.synchronize()
            ms.append((time.perf_counter() - w0) * 1e3)
        tsec = float(np.median(ms)) / 1e3
        # CPU restatement: a few entries at regular 6 / radial 21, per node
        creg, crad = 6, 21
        cn = (2 ** dim) * (6 if dim == 3 else 2) * creg ** (dim - 1) * \
            len(TB.tanh_sinh_fast_rule(crad)[0])
        sample = ids[:: max(1, len(ids) // 4)][:4]
        tp, _, axes = TB.entry_geometry(t, sample)
        c0 = time.perf_counter()
        DO.entry_values(dim, q, 1.0, "laplace" if k is None else "helmholtz", tp, axes,
                        creg, crad, k=k or 0.0)
        csec = time.perf_counter() - c0
        out[name] = {"entries": int(len(ids)), "nodes_per_entry": int(nodes_per_entry),
                     "build_s": tsec, "entries_per_s": len(ids) / tsec,
                     "node_evals_per_s": len(ids) * nodes_per_entry / tsec,
                     "cpu_node_evals_per_s": len(sample) * cn / csec,
                     "cpu_sample": f"{len(sample)} entries at regular {creg} / radial {crad}, "
                                   f"{csec:.2f} s (numpy restatement, 1 core)"}
    head = out["lap3d_q4"]
    hbm, bf16, peak_kind = peaks()
    fp64_peak = measured_fp64_gflops()
    # FP64 flops per enumerated node of the 3D Laplace q=4 build: DADD + DMUL +
    # 2 x DFMA thread instructions of one launch (ncu counters) over its nodes,
    # the nodes of empty sub-boxes included
    ops_per_node = 10.74
    line = {
        "metric": "table build: entries/s (FP64 Duffy radial, default orders)",
        "value": head["entries_per_s"], "unit": "entries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["build_s"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "duffy_table_lap3d_q4", "regular_quad_order": reg,
                   "radial_quad_order": rad, "radial_rule": "tanh-sinh-fast",
                   "l2": "node rules are kB; entries read once"},
        "tables": out,
        "roofline": {"bound": "fp64", "achieved": head["node_evals_per_s"] * ops_per_node / 1e9,
                     "peak": fp64_peak, "unit": "GFLOP/s",
                     "frac": head["node_evals_per_s"] * ops_per_node / 1e9 / fp64_peak,
                     "traffic": None, "peak_source": "cuBLAS DGEMM measured in this run",
                     "fp64_flops_per_node_ncu": ops_per_node},
        "cpu_baseline": {"value": head["cpu_node_evals_per_s"] / head["nodes_per_entry"],
                         "unit": "entries/s", "cores": 1, "kind": "port",
                         "sample": head["cpu_sample"]},
        "e2e": {"value": head["entries_per_s"], "unit": "entries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": head["entries"] * 8,
                "note": "timed around the Python build call (geometry, upload, kernel, "
                        "read-back)"},
        "gpu_launches": args.steps * len(cases),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def csr_main(args):
    """List-1 CSR on the GPU (``vl1_list1_csr``) against the host builder:
    the C2 adaptive octree (23,087 leaves) and a uniform level-6 octree
    (262,144 leaves).  One step = one device build (CUDA events; includes the
    upload of the box arrays and the read-back of the entry count)."""
    import torch

    from volumential_gb300 import workloads as W
    from volumential_gb300.tree_build import (
        build_list1_traversal,
        build_list1_traversal_device,
        build_uniform_tree,
    )

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    out = {}
    for name, tree in (("c2_adaptive_octree", W.config_c2(tables="synthetic").tree),
                       ("uniform_octree_l6", build_uniform_tree(3, 6, 2))):
        t0 = time.perf_counter()
        h = build_list1_traversal(tree)
        host_s = time.perf_counter() - t0
        for _ in range(args.warmup):
            build_list1_traversal_device(tree, as_numpy=False)
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            d = build_list1_traversal_device(tree, as_numpy=False)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        same = bool(np.array_equal(h.neighbor_source_boxes_lists,
                                   d.neighbor_source_boxes_lists.cpu().numpy()) and
                    np.array_equal(h.neighbor_source_boxes_starts,
                                   d.neighbor_source_boxes_starts.cpu().numpy()))
        out[name] = {"leaves": int(len(tree.leaf_boxes)), "nnz": int(h.nnz),
                     "device_ms": float(np.median(ms)), "host_s": host_s,
                     "speedup": host_s * 1e3 / float(np.median(ms)), "equal_to_host": same}
    head = out["uniform_octree_l6"]
    line = {
        "metric": "list-1 CSR build: target boxes/s", "value": head["leaves"] /
        (head["device_ms"] / 1e3), "unit": "boxes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["device_ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": "list1_csr_uniform_octree_l6", "l2": "n/a (one build)"},
        "trees": out,
        "cpu_baseline": {"value": head["leaves"] / head["host_s"], "unit": "boxes/s",
                         "cores": 1, "kind": "port",
                         "sample": "the host builder (numpy) on the same tree"},
        "e2e": {"value": head["leaves"] / (head["device_ms"] / 1e3), "unit": "boxes/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 8},
        "gpu_launches": args.steps * 4,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def tree_main(args):
    """Tree construction on the GPU (refinement criterion evaluated on the
    device, ``vl1_tree_balance``, ``vl1_tree_build_*`` and the list-1 CSR,
    ``vl1_list1_csr``) against the host builder, for the C2 octree: 3D, q=4,
    refined where the variation of the 16-Gaussian density over a leaf's 64
    nodes exceeds 1e-3, levels 2..6, 2:1 balanced.  One step = one device
    build of the tree and its list 1 (CUDA events around the whole call)."""
    import torch

    from volumential_gb300 import workloads as W
    from volumential_gb300.tree_build import (build_adaptive_tree,
                                              build_adaptive_tree_device,
                                              build_list1_traversal,
                                              build_list1_traversal_device)

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    rng = np.random.default_rng(2006)
    mix = W.random_gaussian_mixture(rng, 3, 16, (0.01, 0.08))

    def refine_host(nodes):
        v = mix(nodes)
        return (v.max(axis=-1) - v.min(axis=-1)) > 1e-3

    def refine_dev(nodes):
        v = mix.on_device(nodes)
        return (v.amax(dim=-1) - v.amin(dim=-1)) > 1e-3

    t0 = time.perf_counter()
    host = build_adaptive_tree(3, 4, refine_host, max_level=6, min_level=2)
    hc = build_list1_traversal(host)
    host_s = time.perf_counter() - t0

    def dev_build():
        t = build_adaptive_tree_device(3, 4, refine_dev, max_level=6, min_level=2,
                                       as_numpy=False)
        return t, build_list1_traversal_device(t, as_numpy=False)

    for _ in range(max(1, args.warmup)):
        dev_build()
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        e0.record()
        t, dc = dev_build()
        e1.record()
        e1.synchronize()
        ms.append((time.perf_counter() - w0) * 1e3)
    n_leaves = int(t.leaf_boxes.numel())
    same = (n_leaves == len(host.leaf_boxes) and
            np.array_equal(t.box_levels.cpu().numpy(), host.box_levels) and
            np.array_equal(dc.neighbor_source_boxes_lists.cpu().numpy(),
                           hc.neighbor_source_boxes_lists))
    tms = float(np.median(ms))
    line = {
        "metric": "adaptive tree + list-1 build: leaves/s", "value": n_leaves / (tms / 1e3),
        "unit": "leaves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64/int32", "data": "synthetic",
        "config": {"workload": "tree_c2_adaptive_octree_q4", "leaves": n_leaves,
                   "boxes": int(t.nboxes), "points": int(t.targets.shape[1]),
                   "list1_box_pairs": int(dc.nnz), "l2": "n/a (one build)"},
        "equal_to_host_build": bool(same),
        "cpu_baseline": {"value": len(host.leaf_boxes) / host_s, "unit": "leaves/s",
                         "cores": 1, "kind": "port",
                         "sample": f"the host builder (numpy) on the same tree: {host_s:.2f} s"},
        "e2e": {"value": n_leaves / (tms / 1e3), "unit": "leaves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0, "note": "wall time of the device build call"},
        "gpu_launches": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def split_main(args):
    """Helmholtz split correction (``vl1_split_correction``): the list-1 sum
    of density x weight x R(r), R = G_k - G_0 by its series, over the C3 tree
    (2D uniform level 6, q = 5, 102,400 points, k = 20).  One step = one
    device sum (CUDA events); roofline: the FP64 pipe (per pair 4 flops per
    series term for the two real Horner sums of a real wave number, ~40 for
    the log and the complex accumulation) against the DGEMM rate measured in
    the same run."""
    import torch

    from volumential_gb300 import workloads as W
    from volumential_gb300.batch import tree_arrays
    from volumential_gb300.helmholtz_split import (max_neighbor_distance, series_terms,
                                                   split_correction)

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    k = 20.0
    w = W.config_c3()
    tree = w.tree
    view, keep = tree_arrays(w)
    rng = np.random.default_rng(7)
    wts = torch.from_numpy(rng.standard_normal(tree.ntargets)).to("cuda")
    pts = torch.from_numpy(np.ascontiguousarray(tree.targets)).to("cuda")
    n_terms = series_terms(2, k, max_neighbor_distance(tree))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(3, args.warmup)):
        out = split_correction(view, pts, wts, k, n_terms)
    torch.cuda.synchronize()
    ms = []
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = split_correction(view, pts, wts, k, n_terms)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    clock_info = clocks.stop()
    t = float(np.median(ms)) / 1e3
    pairs = w.pair_count()
    flops = pairs * (4 * n_terms + 40)
    fp64_peak = measured_fp64_gflops()
    # CPU restatement on a sample of target boxes (closed form, numpy)
    from oracle import split_oracle as SO
    tr = w.traversal
    sel = np.arange(0, len(tr.target_boxes), max(1, len(tr.target_boxes) // 64))
    st = tr.neighbor_source_boxes_starts
    sub_starts = np.concatenate([[0], np.cumsum(st[sel + 1] - st[sel])])
    sub_lists = np.concatenate([tr.neighbor_source_boxes_lists[st[i]:st[i + 1]] for i in sel])
    ta = time.perf_counter()
    ref = SO.split_sum(2, k, tree.targets, wts.cpu().numpy().astype(np.complex128),
                       tr.target_boxes[sel], sub_starts, sub_lists, tree.box_target_starts,
                       tree.box_target_counts_nonchild, exclude_self=True)
    cpu_s = time.perf_counter() - ta
    got = out.cpu().numpy()
    mask = ref != 0
    err = float(np.linalg.norm(got[mask] - ref[mask]) / np.linalg.norm(ref[mask]))
    sub_pairs = sum(int(tree.box_target_counts_nonchild[tr.target_boxes[i]]) *
                    int(tree.box_target_counts_nonchild[tr.neighbor_source_boxes_lists[j]])
                    for i in sel for j in range(st[i], st[i + 1]))
    line = {
        "metric": "Helmholtz split correction: point pairs/s", "value": pairs / t,
        "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "split_c3_tree_2d_k20", "points": int(tree.ntargets),
                   "point_pairs": int(pairs), "series_terms": int(n_terms),
                   "l2": "flushed between steps (256 MiB write)"},
        "roofline": {"bound": "fp64", "achieved": flops / t / 1e9, "peak": fp64_peak,
                     "unit": "GFLOP/s", "frac": flops / t / 1e9 / fp64_peak,
                     "kernel": "split_remainder_kernel", "traffic": None,
                     "peak_note": "cuBLAS DGEMM measured in this run"},
        "rel_l2_vs_cpu_closed_form": err,
        "cpu_baseline": {"value": sub_pairs / cpu_s, "unit": "pairs/s", "cores": 1,
                         "kind": "port", "sample": f"{len(sel)} target boxes, closed form "
                                                   "(numpy, oracle/split_oracle.py)"},
        "e2e": None, "clocks": clock_info, "gpu_launches": args.steps,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "c4":
        return c4_main(args)
    if args.workload == "c5":
        return c5_main(args)
    if args.workload == "split":
        return split_main(args)
    if args.workload == "table":
        return table_main(args)
    if args.workload == "csr":
        return csr_main(args)
    if args.workload == "tree":
        return tree_main(args)
    return gb300_main(args)


if __name__ == "__main__":
    sys.exit(main())
