"""Serving: continuous batching of list-1 requests on one GPU.

A request is one right-hand side of one resident problem (a tree and a table
set, e.g. "3D Helmholtz k=12, q=4, uniform level 3").  The engine keeps
trees, plans (tables and tensor-core operands) and schedules resident in HBM
under a byte budget, evicting the least recently used idle entries when a
new one must be admitted.  Each step takes every pending request (up to a
cap) into one batch: ``vl1_batch_update`` re-targets a persistent batch
buffer to the step's problems without allocating, and ``vl1_batch_eval``
runs the batched preparation kernels and one persistent tensor-core launch
per kernel shape.  Two steps are kept in flight so that the host assembles
step k+1 while the GPU runs step k.

Each request is its own batch problem with its own schedule instance (the
tile arrays are shared per resident entry), so its work items, and hence its
result bits, do not depend on what else is in the step: a result is the same
alone and in any mix.

The reference evaluates one problem per ``NearFieldFromCSR`` call
(``expansion_wrangler_fpnd.py:3417-3442``) with a blocking ``queue.finish()``
(``list1.py:1481``); serving many small problems that way is launch- and
synchronisation-bound.
"""

from __future__ import annotations

import collections
import contextlib
import copy
import ctypes as C
import gc
import time

import numpy as np

from . import _lib
from .batch import _plan_from, _plan_kwargs, tree_arrays
from .batched import MixedSchedule

__all__ = ["AdmissionError", "ResidentBudget", "Request", "ServingEngine", "latency_stats"]


class AdmissionError(RuntimeError):
    """A resident entry does not fit the HBM budget even after evicting
    every idle entry."""


def _tensor_bytes(obj):
    import torch

    if isinstance(obj, torch.Tensor):
        return int(obj.numel() * obj.element_size())
    if isinstance(obj, dict):
        return sum(_tensor_bytes(v) for v in obj.values())
    if isinstance(obj, (list, tuple)):
        return sum(_tensor_bytes(v) for v in obj)
    return 0


class ResidentBudget:
    """Byte accounting of resident entries with LRU eviction of idle ones.

    ``admit(key, nbytes, build)`` makes ``key`` resident: entries not in use
    (``pin`` count 0) are evicted oldest first until ``nbytes`` fits, then
    ``build()`` is called and its value stored.  ``release_fn(value)`` frees
    an evicted entry.  Host-only logic (tested without a GPU).
    """

    def __init__(self, budget_bytes, release_fn=None):
        self.budget = int(budget_bytes)
        self.used = 0
        self.entries = collections.OrderedDict()   # key -> [value, nbytes, pins]
        self.release_fn = release_fn
        self.evictions = 0

    def __contains__(self, key):
        return key in self.entries

    def get(self, key):
        e = self.entries[key]
        self.entries.move_to_end(key)
        return e[0]

    def pin(self, key):
        self.entries[key][2] += 1

    def unpin(self, key):
        self.entries[key][2] -= 1

    def _evict_for(self, nbytes):
        for key in list(self.entries):
            if self.used + nbytes <= self.budget:
                break
            value, nb, pins = self.entries[key]
            if pins > 0:
                continue
            del self.entries[key]
            self.used -= nb
            self.evictions += 1
            if self.release_fn:
                self.release_fn(value)
        return self.used + nbytes <= self.budget

    def make_room(self, nbytes):
        """Evict idle entries until ``nbytes`` more would fit; False if they
        cannot."""
        return int(nbytes) <= self.budget and self._evict_for(int(nbytes))

    def admit(self, key, nbytes, build):
        if key in self.entries:
            return self.get(key)
        nbytes = int(nbytes)
        if nbytes > self.budget or not self._evict_for(nbytes):
            raise AdmissionError(
                f"{key!r} needs {nbytes} bytes; budget {self.budget}, in use {self.used} "
                f"by entries that are busy")
        value = build()
        self.entries[key] = [value, nbytes, 0]
        self.used += nbytes
        return value

    def resize(self, key, nbytes):
        """Record the measured size of a resident entry (after building)."""
        e = self.entries[key]
        self.used += int(nbytes) - e[1]
        e[1] = int(nbytes)


class Request:
    __slots__ = ("rid", "key", "coefs", "out", "arrival", "t_start", "t_done", "step",
                 "slot", "waited_build")

    def __init__(self, rid, key, coefs, out, arrival):
        self.rid, self.key, self.coefs, self.out = rid, key, coefs, out
        self.arrival = arrival
        self.t_start = self.t_done = None
        self.step = None
        self.slot = None
        self.waited_build = False   # its table set was being built when it arrived

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


class _Sched:
    """A resident schedule base of one (tree, table level structure) and its
    pool of per-request schedule instances."""

    def __init__(self, key, tree_key, base, ws_bytes):
        self.key, self.tree_key, self.base, self.ws_bytes = key, tree_key, base, ws_bytes
        self.free = []
        self.n_slots = 0


class ServingEngine:
    """Continuous batching over resident problems.

    ``hbm_budget_bytes`` bounds the resident trees, plans and schedules
    (``step_capacity_bytes`` more is held by the batch buffer);
    ``max_step_requests`` caps the requests of one step.  ``register(key,
    workload, table_key)`` declares a problem (built lazily, on its first
    request or by ``admit``); plans are shared by problems with the same
    ``table_key``.

    A problem registered with ``build_tables`` (a function returning its
    table set, e.g. the FP64 Duffy builder for its wave number) has no table
    values yet: the first request for it starts the build on a worker thread
    and its own lowest-priority CUDA stream, and the engine keeps serving the
    other problems meanwhile.  Give the engine a high-priority ``stream``
    (``torch.cuda.Stream(priority=-1)``) and cap the build's grid (the
    ``max_ctas`` of the Duffy builder, e.g. a quarter of the SMs): a step's
    tensor-core CTA needs a whole SM's shared memory, and an SM that keeps
    taking the build's small CTAs never frees it, so an uncapped build holds
    the steps back until it ends.  The request waits (in order) until the
    tables are built, then the plan is admitted like any other.  Built table sets stay in a host
    cache (host memory, outside the HBM budget), so a plan evicted from HBM
    is rebuilt from them without a new table build.
    """

    def __init__(self, *, hbm_budget_bytes, step_capacity_bytes=1 << 30,
                 max_step_requests=128, max_keys_per_item=None, max_inflight=2,
                 stream=None):
        import torch

        self.torch = torch
        self.lib = _lib.lib()
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        self.max_step_requests = int(max_step_requests)
        self.step_capacity = int(step_capacity_bytes)
        self.max_keys_per_item = max_keys_per_item
        self.max_inflight = int(max_inflight)
        self.specs = {}         # key -> (workload, table_key)
        # resident entries share one budget: ("plan", table_key) -> Plan,
        # ("tree", tree_key) -> (view, keep), ("sched", sched_key) -> _Sched;
        # in-flight requests pin the three entries of their problem and a
        # schedule pins its tree
        self.budget = ResidentBudget(hbm_budget_bytes, release_fn=self._release)
        self.pending = collections.deque()
        self.inflight = collections.deque()   # (event, requests)
        self.batch = None
        self.n_steps = 0
        self.step_sizes = []
        self.cold_admissions = 0
        self._next_rid = 0
        # table sets built on demand: host cache, builds in flight, stats
        self._tables = {}           # table_key -> built table set
        self._table_builders = {}   # table_key -> build function
        self._building = {}         # table_key -> Future of a build in flight
        self._plan_args = {}        # table_key -> host arguments of its plan
        self._builder = None
        self._build_stream = None
        self.table_builds = 0
        self.table_build_s = 0.0
        # host seconds spent assembling and launching steps, and device
        # milliseconds of the finished steps (CUDA events around each step)
        self.host_s = 0.0
        self.gpu_ms = 0.0

    # ---- residents -----------------------------------------------------

    def register(self, key, workload, table_key, tree_key=None, sched_key=None,
                 build_tables=None):
        """Declare problem ``key``: ``workload`` (tree, tables, kernel, q);
        problems with the same ``table_key`` share a plan, with the same
        ``tree_key`` a tree, and with the same ``sched_key`` (tree plus table
        level structure and shape) a schedule.  ``build_tables()``, if given,
        returns the table set (``workload.tables`` is then unused) and runs
        on the engine's build thread when the tables are first needed."""
        tree_key = key if tree_key is None else tree_key
        sched_key = (tree_key, table_key) if sched_key is None else sched_key
        self.specs[key] = (workload, table_key, tree_key, sched_key)
        if build_tables is not None:
            self._table_builders.setdefault(table_key, build_tables)

    # ---- table sets built on demand ------------------------------------

    def _run_build(self, fn):
        torch = self.torch
        t0 = time.perf_counter()
        with torch.cuda.stream(self._build_stream):
            tables = fn()
            torch.cuda.current_stream().synchronize()
        return tables, time.perf_counter() - t0

    def _tables_ready(self, key):
        """True when problem ``key`` has its table values; otherwise its
        build is started (once) and False is returned."""
        table_key = self.specs[key][1]
        fn = self._table_builders.get(table_key)
        if fn is None or table_key in self._tables:
            return True
        fut = self._building.get(table_key)
        if fut is None:
            if self._builder is None:
                import concurrent.futures

                self._builder = concurrent.futures.ThreadPoolExecutor(max_workers=1)
                # the lowest priority: the engine's steps (on a higher-priority
                # stream) take free SMs ahead of the build's CTAs
                self._build_stream = self.torch.cuda.Stream(priority=0)
            self._building[table_key] = self._builder.submit(self._run_build, fn)
            return False
        if not fut.done():
            return False
        tables, secs = fut.result()   # a failed build raises here
        del self._building[table_key]
        self._tables[table_key] = tables
        self.table_builds += 1
        self.table_build_s += secs
        return True

    def _build_plan(self, table_key, workload):
        """A new device plan of ``table_key``.  The host arguments (the
        wrangler's payload: compact table, case metadata, normalisers) are
        assembled once per table set and kept in host memory, so a plan
        evicted from HBM is rebuilt with uploads and device kernels only."""
        args = self._plan_args.get(table_key)
        if args is None:
            args = self._plan_args[table_key] = _plan_kwargs(workload)
        nf, kw = args
        return _plan_from(nf, kw, False)

    def _workload(self, key):
        workload, table_key = self.specs[key][:2]
        if table_key not in self._table_builders:
            return workload
        w = copy.copy(workload)
        w.tables = self._tables[table_key]
        return w

    def _release(self, value):
        if isinstance(value, _Sched):
            self.budget.unpin(("tree", value.tree_key))
            value.free.clear()
        elif isinstance(value, tuple):   # (view, keep) of a tree
            pass
        else:
            # an idle plan: its steps ran on the engine's stream and have
            # completed, so no device-wide synchronisation is needed
            value.release(self.stream.cuda_stream)

    def _entry(self, ekey, estimate, build, measure):
        """Admit one entry: room for ``estimate`` bytes, ``build()``, then
        the measured size."""
        if ekey in self.budget:
            return self.budget.get(ekey)
        if not self.budget.make_room(estimate):
            raise AdmissionError(f"{ekey!r}: no room in the HBM budget (entries busy)")
        value = build()
        try:
            self.budget.admit(ekey, measure(value), lambda: value)
        except AdmissionError:
            self._release(value)
            raise
        self.cold_admissions += 1
        return value

    def admit(self, key):
        """Make problem ``key`` resident: its plan, tree and schedule (each
        built if needed, evicting idle entries to stay in the budget).
        Returns (plan, (view, keep), _Sched)."""
        _, table_key, tree_key, sched_key = self.specs[key]
        if not self._tables_ready(key):
            self._building[table_key].result()   # admit() waits for the build
            self._tables_ready(key)
        workload = self._workload(key)
        pkey, tkey, skey = ("plan", table_key), ("tree", tree_key), ("sched", sched_key)
        # pin each entry as soon as it is resident so that admitting the
        # next one cannot evict it
        plan = self._entry(pkey, 1 << 20, lambda: self._build_plan(table_key, workload),
                           lambda pl: pl.device_bytes())
        self.budget.pin(pkey)
        try:
            tree = self._entry(tkey, workload.tree.ntargets * 24,
                               lambda: tree_arrays(workload), lambda t: _tensor_bytes(t[1]))
            self.budget.pin(tkey)
            try:
                def build_sched():
                    view, keep = tree
                    base = MixedSchedule(plan, view, keep, 1, self.stream.cuda_stream,
                                         self.max_keys_per_item, workspace=False)
                    ws = int(self.lib.vl1_mixed_workspace_bytes(plan.handle, C.byref(view), 1))
                    self.budget.pin(tkey)   # held by the schedule while it is resident
                    return _Sched(sched_key, tree_key, base, ws)

                sched = self._entry(skey, workload.tree.ntargets * 4, build_sched,
                                    lambda sc: _tensor_bytes(
                                        [sc.base.tile_rows, sc.base.tile_key_start,
                                         sc.base.key_ids, sc.base.key_xrow, sc.base.items,
                                         sc.base.split_counters, sc.base.split_partials]))
            finally:
                self.budget.unpin(tkey)
        finally:
            self.budget.unpin(pkey)
        return plan, tree, sched

    def _pin_problem(self, key, delta):
        _, table_key, tree_key, sched_key = self.specs[key]
        for ek in (("plan", table_key), ("tree", tree_key), ("sched", sched_key)):
            self.budget.entries[ek][2] += delta

    def _slot(self, sched, plan, tree):
        if sched.free:
            return sched.free.pop()
        sched.n_slots += 1
        view, keep = tree
        s = MixedSchedule(plan, view, keep, 1, self.stream.cuda_stream,
                          self.max_keys_per_item, base=sched.base, workspace=False)
        ek = ("sched", sched.key)
        extra = _tensor_bytes([s.items, s.split_counters, s.split_partials])
        self.budget.make_room(extra)   # best effort: the problem's own entries are pinned
        self.budget.resize(ek, self.budget.entries[ek][1] + extra)
        return s

    # ---- requests ------------------------------------------------------

    def submit(self, key, coefs, out=None, arrival=None):
        """Queue one right-hand side ``coefs`` (CUDA float64 [N]) of problem
        ``key``; ``out`` (optional) receives the result."""
        torch = self.torch
        if coefs.dtype != torch.float64 or not coefs.is_cuda or not coefs.is_contiguous():
            raise TypeError("request densities must be contiguous CUDA float64 tensors")
        req = Request(self._next_rid, key, coefs, out,
                      time.perf_counter() if arrival is None else arrival)
        self._next_rid += 1
        req.waited_build = not self._tables_ready(key)
        self.pending.append(req)
        return req

    def _launch_step(self):
        torch = self.torch
        t_host = time.perf_counter()
        reqs, probs, need = [], [], 0
        waiting = []   # requests whose table set is still being built
        while self.pending and len(reqs) < self.max_step_requests:
            req = self.pending[0]
            if not self._tables_ready(req.key):
                waiting.append(self.pending.popleft())
                continue
            try:
                plan, tree, sched = self.admit(req.key)
            except AdmissionError:
                # the budget is held by this step's and the in-flight steps'
                # problems: the request waits for them to finish
                if reqs or self.inflight:
                    break
                raise
            add = (sched.ws_bytes + 255) // 256 * 256 + 4096
            if reqs and need + add > self.step_capacity // 2:
                break
            self.pending.popleft()
            need += add
            view, keep = tree
            n_points = int(view.n_particles)
            if req.coefs.numel() != n_points:
                raise ValueError(f"request {req.rid}: {req.coefs.numel()} densities for a "
                                 f"tree of {n_points} points")
            if req.out is None:
                req.out = torch.empty(n_points, dtype=torch.complex128 if plan.complex_table
                                      else torch.float64, device="cuda")
            self._pin_problem(req.key, 1)
            req.slot = (sched, self._slot(sched, plan, tree))
            reqs.append(req)
            p = _lib.BatchProblem()
            p.plan = plan.handle
            p.tree = C.cast(C.pointer(view), C.c_void_p)
            p.schedule = C.cast(C.pointer(req.slot[1].c_struct), C.c_void_p)
            p.coefs = req.coefs.data_ptr()
            p.nrhs = 1
            p.result = req.out.data_ptr()
            p.host_items = req.slot[1].items_np.ctypes.data
            probs.append(p)
        if waiting:
            self.pending.extendleft(reversed(waiting))
        if not reqs:
            return False
        arr = (_lib.BatchProblem * len(probs))(*probs)
        sh = C.c_void_p(self.stream.cuda_stream)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev0.record(self.stream)
        if self.batch is None:
            opt = _lib.BatchOptions(0, self.step_capacity)
            h = C.c_void_p()
            _lib.check(self.lib.vl1_batch_create(len(probs), arr, C.byref(opt), C.byref(h)),
                       "vl1_batch_create")
            self.batch = h
        else:
            _lib.check(self.lib.vl1_batch_update(self.batch, len(probs), arr, sh),
                       "vl1_batch_update")
        now = time.perf_counter()
        for q in reqs:
            q.t_start = now
            q.step = self.n_steps
        _lib.check(self.lib.vl1_batch_eval(self.batch, sh), "vl1_batch_eval")
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(self.stream)
        self.inflight.append((ev, reqs, arr, ev0))
        self.n_steps += 1
        self.step_sizes.append(len(reqs))
        self.host_s += time.perf_counter() - t_host
        return True

    def _complete(self, reqs):
        now = time.perf_counter()
        for q in reqs:
            q.t_done = now
            sched, inst = q.slot
            sched.free.append(inst)
            q.slot = None
            self._pin_problem(q.key, -1)

    def poll(self):
        """Retire finished steps; returns the requests completed."""
        done = []
        while self.inflight and self.inflight[0][0].query():
            ev, reqs, _, ev0 = self.inflight.popleft()
            self.gpu_ms += ev0.elapsed_time(ev)
            self._complete(reqs)
            done.extend(reqs)
        return done

    def pump(self):
        """One scheduling round: retire finished steps, launch one if there
        is room in flight and requests are pending."""
        done = self.poll()
        if self.pending and len(self.inflight) < self.max_inflight:
            if not self._launch_step() and not self.inflight:
                time.sleep(50e-6)   # only requests waiting for table builds
        return done

    def drain(self):
        out = []
        with _no_cyclic_gc():
            while self.pending or self.inflight:
                out.extend(self.pump())
        return out

    def check_status(self):
        """Raise if any resident plan's device status word is set."""
        for k, e in self.budget.entries.items():
            if isinstance(k, tuple) and k and k[0] == "plan":
                e[0].raise_on_status(self.stream.cuda_stream)

    def run(self, arrivals):
        """Drive the engine with ``arrivals``: (offset seconds, key, coefs[,
        out]) sorted by time; requests enter the queue at their offset from
        the start.  Returns the requests (with latencies) and the wall time."""
        reqs = []
        with _no_cyclic_gc():
            t0 = time.perf_counter()
            i = 0
            n = len(arrivals)
            while i < n or self.pending or self.inflight:
                now = time.perf_counter() - t0
                while i < n and arrivals[i][0] <= now:
                    a = arrivals[i]
                    reqs.append(self.submit(a[1], a[2], out=a[3] if len(a) > 3 else None,
                                            arrival=t0 + a[0]))
                    i += 1
                self.pump()
            self.torch.cuda.synchronize()
            return reqs, time.perf_counter() - t0

    def close(self):
        while self.inflight:
            self.inflight[0][0].synchronize()
            self.poll()
        if self._builder is not None:
            self._builder.shutdown(wait=True)
            self._builder = None
        if self.batch is not None:
            self.lib.vl1_batch_destroy(self.batch)
            self.batch = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@contextlib.contextmanager
def _no_cyclic_gc():
    """The serving loops run without Python's cyclic garbage collector: a
    full collection over the resident problems' objects stalls the loop for
    tens of milliseconds (it showed as a p99 of ~50 ms in open-loop runs).
    Reference counting still frees the per-request objects."""
    was = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if was:
            gc.enable()


def latency_stats(reqs):
    lat = np.array([q.latency for q in reqs if q.latency is not None]) * 1e3
    if lat.size == 0:
        return {}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "n": int(lat.size)}
