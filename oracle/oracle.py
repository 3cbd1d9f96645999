"""ctypes front end of the C oracle (``oracle/near_field_oracle.c``).

TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` import this module; the product package never
does.  It compiles the oracle with gcc (``build()``), and exposes:

* :func:`full_map`   -- (row, sign) of every (case, source mode, target point)
* :func:`near_field` -- the restated ``near_field`` kernel of
  ``volumential/list1.py:1050-1159`` on numpy inputs (OpenMP over target boxes)

Inputs follow the reference's argument names (``list1.py:1260-1354``).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "near_field_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

_lib = None


def build(force=False):
    """Compile the oracle shared library next to its source."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-std=c11", "-shared", "-fPIC", SRC, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


class Params(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("q", C.c_int32), ("n_tables", C.c_int32),
        ("n_entries", C.c_int32), ("n_cases", C.c_int32),
        ("table_is_complex", C.c_int32), ("coef_is_complex", C.c_int32),
        ("table_data", C.c_void_p), ("mode_nmlz", C.c_void_p),
        ("case_indices", C.c_void_p),
        ("n_case_codes", C.c_int32), ("encoding_base", C.c_int32),
        ("encoding_shift", C.c_double), ("case_encoding_bias", C.c_double),
        ("case_orbit_ranks", C.c_void_p), ("case_axis_perm", C.c_void_p),
        ("case_axis_sign", C.c_void_p), ("case_axis_group", C.c_void_p),
        ("case_value_offsets", C.c_void_p), ("n_orbits", C.c_int32),
        ("axis_sign_power", C.c_void_p), ("axis_direction_signs", C.c_void_p),
        ("direction_sign_axis", C.c_int32),
        ("scaling_exponent", C.c_int32), ("displacement_kind", C.c_int32),
        ("disp_coef", C.c_double), ("table_level_per_level", C.c_int32),
        ("root_extent", C.c_double), ("table_root_extent", C.c_double),
        ("table_starting_level", C.c_int32),
    ]


def _load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        lib.vl1o_near_field.restype = C.c_int
        lib.vl1o_near_field.argtypes = [
            C.POINTER(Params), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
            C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
            C.c_void_p, C.c_int]
        lib.vl1o_full_map.restype = C.c_int
        lib.vl1o_full_map.argtypes = [C.POINTER(Params), C.c_void_p, C.c_void_p]
        lib.vl1o_classify_pairs.restype = C.c_int
        lib.vl1o_classify_pairs.argtypes = [
            C.POINTER(Params), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.vl1o_max_threads.restype = C.c_int
        _lib = lib
    return _lib


def max_threads():
    return int(_load().vl1o_max_threads())


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class OracleProblem:
    """Table payload + policy for the oracle.

    ``metadata`` holds the arithmetic descriptors (the keys of
    ``build_arithmetic_case_metadata``); ``policy`` holds
    ``scaling_exponent``, ``displacement`` ("none" | "log2d"), ``disp_coef`` and
    ``table_level`` ("zero" | "per_level").
    """

    def __init__(self, *, dim, q, table_data, mode_nmlz, case_indices, encoding_base,
                 encoding_shift, metadata, policy, root_extent, table_root_extent,
                 table_starting_level=0, case_encoding_bias=1.0e-10):
        table_data = np.asarray(table_data)
        self.complex_table = np.iscomplexobj(table_data)
        tdt = np.complex128 if self.complex_table else np.float64
        self.table_data = _c(np.atleast_2d(table_data), tdt)
        self.mode_nmlz = _c(np.atleast_2d(mode_nmlz), tdt)
        self.case_indices = _c(case_indices, np.int64)
        self.orbit_ranks = _c(metadata["case_orbit_ranks"], np.uint16)
        self.perm = _c(metadata["case_axis_perm"], np.uint8)
        self.sign = _c(metadata["case_axis_sign"], np.int8)
        self.group = _c(metadata["case_axis_group"], np.uint8)
        self.offsets = _c(metadata["case_value_offsets"], np.int32)
        self.sign_power = _c(metadata["axis_sign_power"], np.uint8)
        self.dir_signs = _c(metadata["axis_direction_signs"], np.int8)
        p = Params()
        p.dim, p.q = int(dim), int(q)
        p.n_tables, p.n_entries = self.table_data.shape
        p.n_cases = self.perm.shape[0]
        p.table_is_complex = int(self.complex_table)
        p.table_data = self.table_data.ctypes.data
        p.mode_nmlz = self.mode_nmlz.ctypes.data
        p.case_indices = self.case_indices.ctypes.data
        p.n_case_codes = self.case_indices.size
        p.encoding_base = int(encoding_base)
        p.encoding_shift = float(encoding_shift)
        p.case_encoding_bias = float(case_encoding_bias)
        p.case_orbit_ranks = self.orbit_ranks.ctypes.data
        p.case_axis_perm = self.perm.ctypes.data
        p.case_axis_sign = self.sign.ctypes.data
        p.case_axis_group = self.group.ctypes.data
        p.case_value_offsets = self.offsets.ctypes.data
        p.n_orbits = self.offsets.size - 1
        p.axis_sign_power = self.sign_power.ctypes.data
        p.axis_direction_signs = self.dir_signs.ctypes.data
        p.direction_sign_axis = int(metadata["direction_sign_axis"])
        p.scaling_exponent = int(policy["scaling_exponent"])
        p.displacement_kind = 1 if policy.get("displacement", "none") == "log2d" else 0
        p.disp_coef = float(policy.get("disp_coef", -0.5 / np.pi))
        p.table_level_per_level = 1 if policy.get("table_level", "zero") == "per_level" else 0
        p.root_extent = float(root_extent)
        p.table_root_extent = float(table_root_extent)
        p.table_starting_level = int(table_starting_level)
        self.params = p

    def full_map(self):
        lib = _load()
        nq = self.params.q ** self.params.dim
        rows = np.empty((self.params.n_cases, nq, nq), dtype=np.int32)
        signs = np.empty((self.params.n_cases, nq, nq), dtype=np.int8)
        st = lib.vl1o_full_map(C.byref(self.params), rows.ctypes.data, signs.ctypes.data)
        if st:
            raise RuntimeError(f"oracle full_map failed with status {st}")
        return rows, signs

    def classify_pairs(self, *, target_boxes, neighbor_source_boxes_starts,
                       neighbor_source_boxes_lists, box_centers, box_levels):
        """(case ids, table levels) of every list-1 pair, in list order, with
        the main loop's FP64 case encoding; case id -1 outside the gallery."""
        lib = _load()
        tb = _c(target_boxes, np.int32)
        st_ = _c(neighbor_source_boxes_starts, np.int32)
        ls = _c(neighbor_source_boxes_lists, np.int32)
        bc = _c(box_centers, np.float64)
        bl = _c(box_levels, np.uint8)
        cases = np.empty(ls.size, dtype=np.int32)
        levels = np.empty(ls.size, dtype=np.int32)
        lib.vl1o_classify_pairs(C.byref(self.params), int(tb.size), tb.ctypes.data,
                                st_.ctypes.data, ls.ctypes.data, int(bc.shape[1]),
                                bc.ctypes.data, bl.ctypes.data, cases.ctypes.data,
                                levels.ctypes.data)
        return cases, levels

    def near_field(self, *, target_boxes, neighbor_source_boxes_starts,
                   neighbor_source_boxes_lists, box_centers, box_levels,
                   box_source_starts, box_source_counts_nonchild, box_target_starts,
                   box_target_counts_nonchild, source_mode_ids, target_point_ids,
                   mode_coefs, nthreads=0, check=True):
        lib = _load()
        coefs = np.asarray(mode_coefs)
        coef_complex = np.iscomplexobj(coefs)
        coefs = _c(coefs, np.complex128 if coef_complex else np.float64)
        out_complex = coef_complex or self.complex_table
        n = int(np.asarray(target_point_ids).size)
        result = np.zeros(n, dtype=np.complex128 if out_complex else np.float64)
        tb = _c(target_boxes, np.int32)
        st_ = _c(neighbor_source_boxes_starts, np.int32)
        ls = _c(neighbor_source_boxes_lists, np.int32)
        bc = _c(box_centers, np.float64)
        bl = _c(box_levels, np.uint8)
        bss = _c(box_source_starts, np.int32)
        bsc = _c(box_source_counts_nonchild, np.int32)
        bts = _c(box_target_starts, np.int32)
        btc = _c(box_target_counts_nonchild, np.int32)
        sm = _c(source_mode_ids, np.int32)
        tm = _c(target_point_ids, np.int32)
        self.params.coef_is_complex = int(coef_complex)
        status = lib.vl1o_near_field(
            C.byref(self.params), int(tb.size), tb.ctypes.data, st_.ctypes.data,
            ls.ctypes.data, int(bc.shape[1]), bc.ctypes.data, bl.ctypes.data,
            bss.ctypes.data, bsc.ctypes.data, bts.ctypes.data, btc.ctypes.data,
            sm.ctypes.data, tm.ctypes.data, coefs.ctypes.data, result.ctypes.data,
            int(nthreads))
        if check and status:
            raise RuntimeError(f"oracle near_field failed with status {status}")
        return result if check else (result, status)


def problem_from_fixture(fx, gallery_mod, orbit_mod):
    """Build an :class:`OracleProblem` from a ``tests/golden/list1_*.npz`` fixture.

    ``gallery_mod``/``orbit_mod`` are the package modules that rebuild the case
    metadata (the fixture stores only the table and the policy).
    """
    dim, q = int(fx["dim"]), int(fx["q"])
    vecs, enc, ci = gallery_mod.generate_list1_gallery(dim)
    base, shift = gallery_mod.gallery_encoding(vecs)

    class _T:
        pass
    t = _T()
    t.dim, t.quad_order, t.n_cases = dim, q, len(vecs)
    t.interaction_case_vecs, t.case_encode, t.case_indices = vecs, enc, ci
    sym = None
    if int(fx["signed"]):
        sym = {"axis_groups": ((0,), tuple(range(1, dim))),
               "axis_sign_power": np.array([1] + [0] * (dim - 1), dtype=np.uint8),
               "axis_direction_signs": np.zeros(dim, dtype=np.int8),
               "direction_sign_axis": -1}
    md = orbit_mod.build_arithmetic_case_metadata(t, sym)
    policy = {"scaling_exponent": int(fx["scaling_exponent"]),
              "displacement": str(fx["displacement"]),
              "disp_coef": float(fx["disp_coef"]),
              "table_level": str(fx["table_level"])}
    return OracleProblem(dim=dim, q=q, table_data=fx["table_data"],
                         mode_nmlz=fx["mode_nmlz"], case_indices=ci,
                         encoding_base=base, encoding_shift=shift, metadata=md,
                         policy=policy, root_extent=float(fx["root_extent"]),
                         table_root_extent=float(fx["table_root_extent"]),
                         table_starting_level=int(fx["table_starting_level"]))
