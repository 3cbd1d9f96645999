"""ctypes binding of ``libvl1.so`` (the C ABI declared in ``include/vl1.h``).

There is no CPU fallback: if the library cannot be loaded, or no CUDA device
is present, every evaluation raises.  The library is built in-tree by
``volumential_gb300._build`` (``__graft_entry__.build()`` calls it).
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import _build

__all__ = ["lib", "PlanDesc", "TreeView", "MixedSchedule", "Status", "VL1Error",
           "VL1TimeoutError", "check", "STATUS_NAMES"]

VL1_OK = 0
VL1_E_INVALID_CASE = 1
VL1_E_ENTRY_OOB = 2
VL1_E_LAYOUT = 3
VL1_E_LEVEL = 4
VL1_E_NONFINITE = 5
VL1_E_UNSUPPORTED_RECON = 6
VL1_E_TIMEOUT = 7
VL1_E_CUDA = 8
VL1_E_ARG = 9
VL1_E_NOMEM = 10
VL1_E_UNSUPPORTED = 11
VL1_NOALLOC_SCRATCH_BYTES = 32 << 20

STATUS_NAMES = {
    VL1_OK: "VL1_OK", VL1_E_INVALID_CASE: "VL1_E_INVALID_CASE",
    VL1_E_ENTRY_OOB: "VL1_E_ENTRY_OOB", VL1_E_LAYOUT: "VL1_E_LAYOUT",
    VL1_E_LEVEL: "VL1_E_LEVEL", VL1_E_NONFINITE: "VL1_E_NONFINITE",
    VL1_E_UNSUPPORTED_RECON: "VL1_E_UNSUPPORTED_RECON",
    VL1_E_TIMEOUT: "VL1_E_TIMEOUT", VL1_E_CUDA: "VL1_E_CUDA", VL1_E_ARG: "VL1_E_ARG",
    VL1_E_NOMEM: "VL1_E_NOMEM", VL1_E_UNSUPPORTED: "VL1_E_UNSUPPORTED",
}

VL1_REAL64 = 0
VL1_COMPLEX128 = 1
VL1_RECON_SCALAR_ARITH = 0
VL1_RECON_SIGNED_ARITH = 1
VL1_RECON_DENSE = 2
VL1_DISP_NONE = 0
VL1_DISP_LOG2D = 1
VL1_LEVEL_ZERO = 0
VL1_LEVEL_PER_LEVEL = 1


class VL1Error(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class VL1TimeoutError(VL1Error, TimeoutError):
    """A bounded device wait gave up (``VL1_E_TIMEOUT``); the call wrote no
    results and the device, the plan and the schedule stay usable."""


class PlanDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("quad_order", C.c_int32), ("n_tables", C.c_int32),
        ("n_table_entries", C.c_int32), ("n_cases", C.c_int32),
        ("n_case_orbits", C.c_int32), ("value_type", C.c_int32),
        ("reconstruction_kind", C.c_int32),
        ("table_data", C.c_void_p), ("mode_nmlz", C.c_void_p),
        ("case_indices", C.c_void_p), ("n_case_codes", C.c_int32),
        ("encoding_base", C.c_int32), ("encoding_shift", C.c_double),
        ("case_encoding_bias", C.c_double),
        ("case_orbit_ranks", C.c_void_p), ("case_axis_perm", C.c_void_p),
        ("case_axis_sign", C.c_void_p), ("case_axis_group", C.c_void_p),
        ("case_value_offsets", C.c_void_p), ("axis_sign_power", C.c_void_p),
        ("axis_direction_signs", C.c_void_p), ("direction_sign_axis", C.c_int32),
        ("scaling_exponent", C.c_int32), ("displacement_kind", C.c_int32),
        ("displacement_coef", C.c_double), ("table_level_kind", C.c_int32),
        ("table_root_extent", C.c_double), ("table_starting_level", C.c_int32),
    ]


class TreeView(C.Structure):
    _fields_ = [
        ("n_target_boxes", C.c_int32), ("target_boxes", C.c_void_p),
        ("neighbor_source_boxes_starts", C.c_void_p),
        ("neighbor_source_boxes_lists", C.c_void_p),
        ("aligned_nboxes", C.c_int64), ("box_centers", C.c_void_p),
        ("box_levels", C.c_void_p), ("box_source_starts", C.c_void_p),
        ("box_source_counts_nonchild", C.c_void_p), ("box_target_starts", C.c_void_p),
        ("box_target_counts_nonchild", C.c_void_p), ("source_mode_ids", C.c_void_p),
        ("target_point_ids", C.c_void_p), ("n_particles", C.c_int64),
        ("nboxes", C.c_int64), ("root_extent", C.c_double),
    ]


class MixedItem(C.Structure):
    _fields_ = [("tile", C.c_int32), ("key_begin", C.c_int32), ("key_end", C.c_int32),
                ("split", C.c_int32), ("part", C.c_int32), ("nparts", C.c_int32),
                ("slot", C.c_int32), ("reserved", C.c_int32)]


class MixedSchedule(C.Structure):
    _fields_ = [
        ("n_tiles", C.c_int32), ("tile_rows", C.c_void_p), ("tile_key_start", C.c_void_p),
        ("key_ids", C.c_void_p), ("key_xrow", C.c_void_p),
        ("n_items", C.c_int32), ("items", C.c_void_p),
        ("n_splits", C.c_int32), ("n_slots", C.c_int32),
        ("split_counters", C.c_void_p), ("split_partials", C.c_void_p),
        ("n_chunks", C.c_int32),
    ]


class BatchProblem(C.Structure):
    _fields_ = [("plan", C.c_void_p), ("tree", C.c_void_p), ("schedule", C.c_void_p),
                ("coefs", C.c_void_p), ("nrhs", C.c_int32), ("result", C.c_void_p),
                ("host_items", C.c_void_p)]


class BatchOptions(C.Structure):
    _fields_ = [("ctas_per_launch", C.c_int32), ("capacity_bytes", C.c_int64)]


class DuffyDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("q", C.c_int32), ("n_entries", C.c_int32),
                ("n_reg", C.c_int32), ("n_rad", C.c_int32), ("kernel", C.c_int32),
                ("complex_output", C.c_int32), ("max_ctas", C.c_int32),
                ("power", C.c_int32), ("derivative", C.c_int32),
                ("extent", C.c_double), ("k", C.c_double),
                ("target_points", C.c_void_p), ("decomposition_targets", C.c_void_p),
                ("mode_axes", C.c_void_p), ("regular_nodes", C.c_void_p),
                ("regular_weights", C.c_void_p), ("radial_nodes", C.c_void_p),
                ("radial_weights", C.c_void_p), ("interp_nodes", C.c_void_p),
                ("interp_weights", C.c_void_p)]


VL1_DUFFY_LAPLACE2D, VL1_DUFFY_LAPLACE3D, VL1_DUFFY_HELMHOLTZ2D = 0, 1, 2
VL1_DUFFY_HELMHOLTZ3D, VL1_DUFFY_CONSTANT, VL1_DUFFY_PLANE_WAVE = 3, 4, 5
VL1_DUFFY_POWER, VL1_DUFFY_POWER_LOG = 6, 7
VL1_SPLIT_REAL_K = 1


class SplitDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("n_points", C.c_int32), ("n_terms", C.c_int32),
                ("exclude_self", C.c_int32), ("weights_complex", C.c_int32),
                ("flags", C.c_int32), ("tree", C.c_void_p), ("points", C.c_void_p),
                ("weights", C.c_void_p), ("coefficients", C.c_void_p),
                ("result", C.c_void_p)]


class CsrDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nboxes", C.c_int32), ("n_leaves", C.c_int32),
                ("max_level", C.c_int32), ("box_levels", C.c_void_p),
                ("box_coords", C.c_void_p), ("leaf_boxes", C.c_void_p),
                ("starts", C.c_void_p), ("lists", C.c_void_p),
                ("lists_capacity", C.c_int64), ("workspace", C.c_void_p),
                ("workspace_bytes", C.c_int64)]


class ScheduleSizes(C.Structure):
    _fields_ = [("n_tiles", C.c_int32), ("n_entries", C.c_int64)]


class Status(C.Structure):
    _fields_ = [("code", C.c_int32), ("count", C.c_int32),
                ("detail0", C.c_int32), ("detail1", C.c_int32)]


# symbol -> (restype, argtypes); the single source of truth for what the
# library must export (checked by the CPU test suite)
SIGNATURES = {
    "vl1_version": (C.c_int32, []),
    "vl1_last_error_string": (C.c_char_p, []),
    "vl1_plan_create": (C.c_int32, [C.POINTER(PlanDesc), C.POINTER(C.c_void_p)]),
    "vl1_plan_destroy": (C.c_int32, [C.c_void_p]),
    "vl1_plan_release": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vl1_eval_fp64": (C.c_int32, [C.c_void_p, C.POINTER(TreeView), C.c_void_p,
                                  C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "vl1_orbit_index_map": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    "vl1_classify_pairs": (C.c_int32, [C.c_void_p, C.POINTER(TreeView), C.c_void_p,
                                       C.c_void_p]),
    "vl1_mixed_workspace_bytes": (C.c_int64, [C.c_void_p, C.POINTER(TreeView), C.c_int32]),
    "vl1_schedule_build_begin": (C.c_int32, [C.c_void_p, C.POINTER(TreeView), C.c_int64,
                                             C.c_int32, C.POINTER(C.c_void_p),
                                             C.POINTER(ScheduleSizes), C.c_void_p]),
    "vl1_schedule_build_key_start": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vl1_schedule_build_fill": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p]),
    "vl1_schedule_builder_destroy": (C.c_int32, [C.c_void_p]),
    "vl1_mixed_work_items": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "vl1_mixed_geometry": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vl1_plan_set_mixed_geometry": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32]),
    "vl1_eval_mixed": (C.c_int32, [C.c_void_p, C.POINTER(TreeView),
                                   C.POINTER(MixedSchedule), C.c_void_p, C.c_int32,
                                   C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "vl1_batch_create": (C.c_int32, [C.c_int32, C.POINTER(BatchProblem),
                                     C.POINTER(BatchOptions), C.POINTER(C.c_void_p)]),
    "vl1_batch_eval": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vl1_set_kernel_events": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vl1_test_set_wait_fault": (C.c_int32, [C.c_int32, C.c_int32]),
    "vl1_duffy_table": (C.c_int32, [C.POINTER(DuffyDesc), C.c_void_p, C.c_void_p]),
    "vl1_split_correction": (C.c_int32, [C.POINTER(SplitDesc), C.c_void_p]),
    "vl1_list1_csr_workspace_bytes": (C.c_int64, [C.c_int32]),
    "vl1_tree_balance": (C.c_int32, [C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.c_void_p,
                                     C.c_void_p, C.c_void_p]),
    "vl1_tree_build_begin": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                         C.c_void_p, C.c_double, C.c_void_p,
                                         C.POINTER(C.c_void_p), C.c_void_p, C.c_void_p]),
    "vl1_tree_build_level_starts": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vl1_tree_build_fill": (C.c_int32, [C.c_void_p] + [C.c_void_p] * 11 + [C.c_void_p]),
    "vl1_tree_builder_destroy": (C.c_int32, [C.c_void_p]),
    "vl1_list1_csr": (C.c_int32, [C.POINTER(CsrDesc), C.POINTER(C.c_int64), C.c_void_p]),
    "vl1_batch_update": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(BatchProblem),
                                     C.c_void_p]),
    "vl1_batch_destroy": (C.c_int32, [C.c_void_p]),
    "vl1_batch_device_bytes": (C.c_int64, [C.c_void_p]),
    "vl1_batch_kernel_launches": (C.c_int32, [C.c_void_p]),
    "vl1_eval_mixed_noalloc": (C.c_int32, [C.c_void_p, C.POINTER(TreeView),
                                           C.POINTER(MixedSchedule), C.c_void_p, C.c_int32,
                                           C.c_void_p, C.c_void_p]),
    "vl1_status_read": (C.c_int32, [C.c_void_p, C.POINTER(Status), C.c_int32,
                                    C.c_void_p]),
    "vl1_plan_device_bytes": (C.c_int64, [C.c_void_p]),
}

_lock = threading.Lock()
_lib = None


def lib():
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not os.path.exists(path) or not _build.up_to_date():
                _build.build()
            handle = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def last_error():
    msg = lib().vl1_last_error_string()
    return msg.decode() if msg else ""


def check(code, what=""):
    if code != VL1_OK:
        raise VL1Error(code, f"{what}: {last_error()}" if what else last_error())


def ptr(x):
    """Raw pointer of a torch tensor / numpy array (None -> NULL)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)!r}")
