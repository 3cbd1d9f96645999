"""Device plans: one per table payload, owned by Python, created through the C ABI.

A plan holds the table, normalizers, orbit descriptors and the expanded
(level, case) blocks in HBM.  ``plan_cache_get`` keeps an LRU of plans keyed
by the identity of the payload arrays, like the wrangler's payload cache of
the reference (``expansion_wrangler_fpnd.py:2880-2881, 3152-3157``).
"""

from __future__ import annotations

import collections
import ctypes as C
import threading

import numpy as np

from . import _lib

__all__ = ["Plan", "plan_cache_get", "tree_view_from_arrays", "as_device_tensor",
           "stream_handle", "require_cuda", "PLAN_CACHE_MAX"]

PLAN_CACHE_MAX = 16
_cache: "collections.OrderedDict" = collections.OrderedDict()
_cache_lock = threading.Lock()


_cuda_ok = False


def require_cuda():
    global _cuda_ok
    import torch
    if not _cuda_ok:
        if not torch.cuda.is_available():
            raise RuntimeError(
                "volumential_gb300 evaluates list 1 on a CUDA device only; no CUDA "
                "device is available (there is no CPU fallback)")
        _cuda_ok = True   # a device, once seen, stays (the query costs microseconds)
    return torch


def as_device_tensor(x, dtype=None):
    """A contiguous CUDA tensor view/copy of ``x`` (numpy, torch, list)."""
    torch = require_cuda()
    if isinstance(x, torch.Tensor):
        t = x
    else:
        if hasattr(x, "get") and not isinstance(x, np.ndarray):
            x = x.get()
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x)))
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    if not t.is_cuda:
        t = t.to("cuda", non_blocking=False)
    if not t.is_contiguous():
        t = t.contiguous()
    return t


def stream_handle(queue):
    """cudaStream_t of ``queue`` (a torch.cuda.Stream) or torch's current stream."""
    torch = require_cuda()
    if queue is None:
        return torch.cuda.current_stream().cuda_stream
    if hasattr(queue, "cuda_stream"):
        return queue.cuda_stream
    if isinstance(queue, int):
        return queue
    raise TypeError("queue must be None or a torch.cuda.Stream")


_views: "collections.OrderedDict" = collections.OrderedDict()
_VIEW_CACHE_MAX = 8


def tree_view_from_arrays(**arrays):
    """Build a ``vl1_tree_view`` from arrays; returns (view, tensors to keep alive).

    When every array is already a CUDA tensor of the kernel's dtype, the view
    is cached per array identity (pointer, shape, dtype and in-place version
    counter), so repeated calls over one tree skip the rebuild."""
    torch = require_cuda()
    key = None
    tensors = [arrays[k] for k in _VIEW_ARGS]
    if all(isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous() for t in tensors):
        key = (tuple(_token(t) for t in tensors), float(arrays["root_extent"]))
        with _cache_lock:
            hit = _views.get(key)
            if hit is not None:
                _views.move_to_end(key)
                return hit
    out = _tree_view_from_arrays(**arrays)
    if key is not None and all(out[1][k] is t for k, t in zip(_VIEW_KEYS, tensors)):
        with _cache_lock:
            _views[key] = out
            while len(_views) > _VIEW_CACHE_MAX:
                _views.popitem(last=False)
    return out


# the array arguments and their keep-dict names, in one order
_VIEW_ARGS = ("target_boxes", "neighbor_source_boxes_starts", "neighbor_source_boxes_lists",
              "box_centers", "box_levels", "box_source_starts", "box_source_counts_nonchild",
              "box_target_starts", "box_target_counts_nonchild", "source_mode_ids",
              "target_point_ids")
_VIEW_KEYS = ("target_boxes", "starts", "lists", "centers", "levels", "src_starts",
              "src_counts", "tgt_starts", "tgt_counts", "smode", "tmode")


def _tree_view_from_arrays(*, target_boxes, neighbor_source_boxes_starts,
                           neighbor_source_boxes_lists, box_centers, box_levels,
                           box_source_starts, box_source_counts_nonchild,
                           box_target_starts, box_target_counts_nonchild,
                           source_mode_ids, target_point_ids, root_extent):
    torch = require_cuda()
    i32 = torch.int32
    keep = {
        "target_boxes": as_device_tensor(target_boxes, i32),
        "starts": as_device_tensor(neighbor_source_boxes_starts, i32),
        "lists": as_device_tensor(neighbor_source_boxes_lists, i32),
        "centers": as_device_tensor(box_centers, torch.float64),
        "levels": as_device_tensor(box_levels, torch.uint8),
        "src_starts": as_device_tensor(box_source_starts, i32),
        "src_counts": as_device_tensor(box_source_counts_nonchild, i32),
        "tgt_starts": as_device_tensor(box_target_starts, i32),
        "tgt_counts": as_device_tensor(box_target_counts_nonchild, i32),
        "smode": as_device_tensor(source_mode_ids, i32),
        "tmode": as_device_tensor(target_point_ids, i32),
    }
    v = _lib.TreeView()
    v.n_target_boxes = int(keep["target_boxes"].numel())
    if keep["starts"].numel() != v.n_target_boxes + 1:
        raise ValueError("neighbor_source_boxes_starts must have n_target_boxes + 1 entries")
    v.target_boxes = keep["target_boxes"].data_ptr()
    v.neighbor_source_boxes_starts = keep["starts"].data_ptr()
    v.neighbor_source_boxes_lists = keep["lists"].data_ptr()
    if keep["centers"].dim() != 2:
        raise ValueError("box_centers must be [dim, aligned_nboxes]")
    v.aligned_nboxes = int(keep["centers"].shape[1])
    v.box_centers = keep["centers"].data_ptr()
    v.box_levels = keep["levels"].data_ptr()
    v.box_source_starts = keep["src_starts"].data_ptr()
    v.box_source_counts_nonchild = keep["src_counts"].data_ptr()
    v.box_target_starts = keep["tgt_starts"].data_ptr()
    v.box_target_counts_nonchild = keep["tgt_counts"].data_ptr()
    v.source_mode_ids = keep["smode"].data_ptr()
    v.target_point_ids = keep["tmode"].data_ptr()
    v.n_particles = int(keep["tmode"].numel())
    v.nboxes = int(keep["levels"].numel())
    v.root_extent = float(root_extent)
    validate_tree_arrays(keep, dim=int(keep["centers"].shape[0]))
    return v, keep


_validated: "collections.OrderedDict" = collections.OrderedDict()


def _token(t):
    return (t.data_ptr(), t._version, tuple(t.shape), str(t.dtype))


def validate_tree_arrays(keep, dim):
    """Bounds of every index the kernels load through (cached per array set).

    The kernels check case codes, box counts against q^dim and mode ids
    themselves; everything else that addresses memory is checked here, so that
    an invalid tree raises on the host and never reaches a device load.
    """
    key = tuple(_token(t) for t in keep.values())
    if key in _validated:
        _validated.move_to_end(key)
        return
    torch = require_cuda()
    nboxes = int(keep["levels"].numel())
    npart = int(keep["tmode"].numel())
    ntb = int(keep["target_boxes"].numel())
    st = keep["starts"]
    ls = keep["lists"]
    if dim not in (2, 3):
        raise ValueError(f"box_centers must have 2 or 3 rows, got {dim}")
    if int(keep["smode"].numel()) != npart:
        raise ValueError("source_mode_ids and target_point_ids must have the same length "
                         "(sources are targets)")
    for name in ("src_starts", "src_counts", "tgt_starts", "tgt_counts"):
        if int(keep[name].numel()) < nboxes:
            raise ValueError(f"box array {name} has fewer than nboxes={nboxes} entries")
    if int(keep["centers"].shape[1]) < nboxes:
        raise ValueError("box_centers has fewer columns than boxes")
    checks = []
    if ntb:
        checks += [st[0] != 0, st[-1] != ls.numel(), (st[1:] < st[:-1]).any(),
                   keep["target_boxes"].min() < 0, keep["target_boxes"].max() >= nboxes]
    if ls.numel():
        checks += [ls.min() < 0, ls.max() >= nboxes]
    if nboxes:
        lv = keep["levels"]
        checks += [lv.max() > 60]
        for s_name, c_name in (("src_starts", "src_counts"), ("tgt_starts", "tgt_counts")):
            s = keep[s_name][:nboxes].to(torch.int64)
            c = keep[c_name][:nboxes].to(torch.int64)
            used = c > 0
            checks += [(used & (s < 0)).any(), (used & (s + c > npart)).any(), (c < 0).any()]
    if checks and bool(torch.stack([torch.as_tensor(x, device="cuda").reshape(())
                                    for x in checks]).any()):
        raise ValueError(
            "invalid list-1 tree arrays: CSR starts must run from 0 to len(lists), box "
            "ids must lie in [0, nboxes), box particle ranges in [0, n_particles) and "
            "levels below 61")
    # the entry holds the validated tensors, so their memory cannot be reused
    # by other arrays while the key is cached
    _validated[key] = dict(keep)
    while len(_validated) > 8:
        _validated.popitem(last=False)


class Plan:
    """Owner of one ``vl1_plan``."""

    def __init__(self, *, dim, quad_order, n_tables, table_data, mode_nmlz, case_indices,
                 encoding_base, encoding_shift, case_encoding_bias, case_orbit_ranks,
                 case_axis_perm, case_axis_sign, case_axis_group, case_value_offsets,
                 axis_sign_power, axis_direction_signs, direction_sign_axis,
                 reconstruction_kind, scaling_exponent, displacement_kind,
                 displacement_coef, table_level_kind, table_root_extent,
                 table_starting_level):
        require_cuda()
        lib = _lib.lib()
        table = np.atleast_2d(np.asarray(table_data))
        self.complex_table = np.iscomplexobj(table)
        vdt = np.complex128 if self.complex_table else np.float64
        self._host = {
            "table": np.ascontiguousarray(table, dtype=vdt),
            "nmlz": np.ascontiguousarray(np.atleast_2d(mode_nmlz), dtype=vdt),
            "case_indices": np.ascontiguousarray(case_indices, dtype=np.int64),
            "ranks": np.ascontiguousarray(case_orbit_ranks, dtype=np.uint16),
            "perm": np.ascontiguousarray(case_axis_perm, dtype=np.uint8),
            "sign": np.ascontiguousarray(case_axis_sign, dtype=np.int8),
            "group": np.ascontiguousarray(case_axis_group, dtype=np.uint8),
            "offsets": np.ascontiguousarray(case_value_offsets, dtype=np.int32),
            "sign_power": np.ascontiguousarray(axis_sign_power, dtype=np.uint8),
            "dir_signs": np.ascontiguousarray(axis_direction_signs, dtype=np.int8),
        }
        h = self._host
        if h["table"].shape[0] != int(n_tables):
            raise ValueError(f"table_data has {h['table'].shape[0]} levels, expected {n_tables}")
        nq = int(quad_order) ** int(dim)
        if h["nmlz"].shape != (int(n_tables), nq):
            raise ValueError(f"mode_nmlz must be [{n_tables}, {nq}], got {h['nmlz'].shape}")
        d = _lib.PlanDesc()
        d.dim, d.quad_order, d.n_tables = int(dim), int(quad_order), int(n_tables)
        d.n_table_entries = int(h["table"].shape[1])
        d.n_cases = int(h["perm"].shape[0])
        d.n_case_orbits = int(h["offsets"].size - 1)
        d.value_type = _lib.VL1_COMPLEX128 if self.complex_table else _lib.VL1_REAL64
        d.reconstruction_kind = int(reconstruction_kind)
        d.table_data = h["table"].ctypes.data
        d.mode_nmlz = h["nmlz"].ctypes.data
        d.case_indices = h["case_indices"].ctypes.data
        d.n_case_codes = int(h["case_indices"].size)
        d.encoding_base = int(encoding_base)
        d.encoding_shift = float(encoding_shift)
        d.case_encoding_bias = float(case_encoding_bias)
        d.case_orbit_ranks = h["ranks"].ctypes.data
        d.case_axis_perm = h["perm"].ctypes.data
        d.case_axis_sign = h["sign"].ctypes.data
        d.case_axis_group = h["group"].ctypes.data
        d.case_value_offsets = h["offsets"].ctypes.data
        d.axis_sign_power = h["sign_power"].ctypes.data
        d.axis_direction_signs = h["dir_signs"].ctypes.data
        d.direction_sign_axis = int(direction_sign_axis)
        d.scaling_exponent = int(scaling_exponent)
        d.displacement_kind = int(displacement_kind)
        d.displacement_coef = float(displacement_coef)
        d.table_level_kind = int(table_level_kind)
        d.table_root_extent = float(table_root_extent)
        d.table_starting_level = int(table_starting_level)
        self.desc = d
        self.dim, self.quad_order, self.nq = int(dim), int(quad_order), nq
        self.n_tables = int(n_tables)
        self.n_cases = d.n_cases
        handle = C.c_void_p()
        _lib.check(lib.vl1_plan_create(C.byref(d), C.byref(handle)), "vl1_plan_create")
        self._handle = handle
        self._lib = lib

    @property
    def handle(self):
        if self._handle is None:
            raise RuntimeError("plan destroyed")
        return self._handle

    def device_bytes(self):
        return int(self._lib.vl1_plan_device_bytes(self.handle))

    def destroy(self):
        if getattr(self, "_handle", None) is not None:
            self._lib.vl1_plan_destroy(self._handle)
            self._handle = None

    def release(self, stream):
        """Free the plan without a device-wide synchronisation, in the order
        of ``stream`` (a cudaStream_t handle): every call using the plan
        must have been issued on that stream or have completed."""
        if getattr(self, "_handle", None) is not None:
            self._lib.vl1_plan_release(self._handle, C.c_void_p(stream))
            self._handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def eval_fp64(self, view, coefs, out, *, stream, nrhs=1):
        """Plain FP64 kernel; ``coefs``/``out`` are CUDA tensors [nrhs*N]."""
        import torch
        if coefs.dtype not in (torch.float64, torch.complex128):
            raise TypeError("coefs must be float64 or complex128")
        ctype = _lib.VL1_COMPLEX128 if coefs.is_complex() else _lib.VL1_REAL64
        n = int(view.n_particles)
        if coefs.numel() != nrhs * n or out.numel() != nrhs * n:
            raise ValueError(f"coefs/result must hold nrhs*n_particles = {nrhs * n} values")
        if not (coefs.is_cuda and out.is_cuda and coefs.is_contiguous() and out.is_contiguous()):
            raise ValueError("coefs and result must be contiguous CUDA tensors")
        st = self._lib.vl1_eval_fp64(self.handle, C.byref(view), coefs.data_ptr(), ctype,
                                     int(nrhs), out.data_ptr(), C.c_void_p(stream))
        _lib.check(st, "vl1_eval_fp64")

    def mixed_geometry(self):
        out = (C.c_int32 * 5)()
        _lib.check(self._lib.vl1_mixed_geometry(self.handle, out), "vl1_mixed_geometry")
        return dict(zip(("kp", "kc", "n_kc", "np", "nch"), list(out)))

    def set_mixed_geometry(self, kc, nch):
        """Tile shape of the tensor-core kernel: ``kc`` source points per
        pipeline unit (16 or 32), ``nch`` output columns per CTA (16, 32 or
        64).  Schedules are cached per shape."""
        _lib.check(self._lib.vl1_plan_set_mixed_geometry(self.handle, int(kc), int(nch)),
                   "vl1_plan_set_mixed_geometry")

    def mixed_shapes(self):
        """The tile shapes (kc, nch) this plan can take."""
        geo = self.mixed_geometry()
        n = self.nq * (2 if self.complex_table else 1)
        out = []
        for kc in (16, 32):
            if kc > geo["kp"]:
                continue
            for nch in (16, 32, 64):
                if nch > 16 and -(-n // 16) * 16 <= nch // 2:
                    continue   # all padding beyond half a chunk
                out.append((kc, nch))
        return out

    def read_status(self, stream=None, reset=True):
        s = _lib.Status()
        _lib.check(self._lib.vl1_status_read(self.handle, C.byref(s), int(reset),
                                             C.c_void_p(stream or 0)), "vl1_status_read")
        return s

    def raise_on_status(self, stream=None):
        """Read and clear the device status; raise the reference's exception type."""
        s = self.read_status(stream)
        if s.code == _lib.VL1_OK:
            return
        if s.code == _lib.VL1_E_LAYOUT:
            raise ValueError(
                "table-based near-field evaluation requires exactly "
                f"{self.nq} quadrature points per active source/target box and box-local "
                f"mode ids in [0, {self.nq}); the kernel found {s.count} violations "
                f"(first at target box {s.detail0}). Build the particle tree from the "
                "mesh box-tree to preserve per-cell quadrature layout.")
        if s.code == _lib.VL1_E_INVALID_CASE:
            raise RuntimeError(
                f"list1 case encoding produced {s.count} codes outside the interaction "
                f"gallery (first at target box {s.detail0}, list position {s.detail1}); "
                "the tree is not 2:1 balanced or box centres are inconsistent")
        if s.code == _lib.VL1_E_TIMEOUT:
            raise _lib.VL1TimeoutError(
                s.code, f"a bounded device wait gave up in {s.count} work items (first: "
                        f"tile {s.detail0}, column chunk {s.detail1}); no results were "
                        "written")
        raise _lib.VL1Error(s.code, f"device status: {s.count} faults, first detail "
                                    f"({s.detail0}, {s.detail1})")

    def orbit_index_map(self, stream=None):
        """Device-computed (rows, signs) of every (case, source mode, target point)."""
        torch = require_cuda()
        rows = torch.empty((self.n_cases, self.nq, self.nq), dtype=torch.int32, device="cuda")
        signs = torch.empty((self.n_cases, self.nq, self.nq), dtype=torch.int8, device="cuda")
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(self._lib.vl1_orbit_index_map(self.handle, rows.data_ptr(),
                                                 signs.data_ptr(), C.c_void_p(s)),
                   "vl1_orbit_index_map")
        return rows, signs


def plan_cache_get(key, **kwargs):
    with _cache_lock:
        plan = _cache.get(key)
        if plan is not None:
            _cache.move_to_end(key)
            return plan
    plan = Plan(**kwargs)
    with _cache_lock:
        _cache[key] = plan
        while len(_cache) > PLAN_CACHE_MAX:
            _, old = _cache.popitem(last=False)
            old.destroy()
    return plan


def clear_plan_cache():
    with _cache_lock:
        while _cache:
            _, p = _cache.popitem(last=False)
            p.destroy()
