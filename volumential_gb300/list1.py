"""List-1 near-field evaluator: ``NearFieldFromCSR`` on GB300.

Drop-in for ``volumential.list1`` (``volumential/list1.py``).  The class
names, constructor arguments, ``extra_kwargs`` handling, scaling-policy
strings and the ``__call__`` keyword arguments follow the reference
(``list1.py:49-437`` and ``:1260-1487``); the evaluation itself runs in the
hand-written CUDA library through the C ABI of ``include/vl1.h``.  There is no
CPU fallback.

Differences from the reference that a caller can see:

* arrays are torch tensors (CUDA tensors are used in place; numpy / CPU
  tensors are copied to the device), and ``queue`` is ``None`` or a
  ``torch.cuda.Stream``;
* ``__call__`` returns ``(result, event)`` with a ``torch.cuda.Event``;
* policy code strings are not compiled: the scaling, displacement and table
  level codes the reference can generate (its inferred rules, the Helmholtz
  split rules of ``expansion_wrangler_fpnd.py:4777-4833`` and the per-level
  rule) are recognised and mapped onto the kernel; other custom strings raise
  ``NotImplementedError``;
* invalid cases (a case code outside the gallery) and layout violations are
  reported by the kernel through a status word and raised as exceptions,
  where the reference would read out of bounds;
* ``list1_precision`` (an extra keyword, default ``"fp64"``) selects the plain
  FP64 kernel or the tensor-core path (``"mixed"``: exact FP16 digit products,
  FP64 sums, relative error ~2^-40 of sum |table| |density|).
"""

from __future__ import annotations

import logging
import math
import numbers
import re
from dataclasses import dataclass

import numpy as np

from . import _lib
from .kernels import base_kernel, kernel_class_name


def _is_scalar(v):
    return isinstance(v, (str, bytes, numbers.Number, np.generic, type(None)))


def _memo_token(v):
    """Key of one extra keyword argument in the policy memo."""
    if isinstance(v, np.generic):
        return (type(v).__name__, v.item())
    if _is_scalar(v):
        return v
    if isinstance(v, (list, tuple, dict)):
        return (type(v).__name__, repr(v))
    return (type(v).__name__, id(v))

logger = logging.getLogger(__name__)

CASE_ENCODING_BIAS_DEFAULT = 1.0e-10

__all__ = ["KernelScalingPolicy", "NearFieldEvalBase", "NearFieldFromCSR",
           "CASE_ENCODING_BIAS_DEFAULT", "parse_policy"]


@dataclass(frozen=True)
class KernelScalingPolicy:
    """Describes how a List 1 evaluator selects and rescales table data."""

    kernel_name: str
    mode: str
    infer_kernel_scaling: bool
    single_table_scaling_supported: bool
    reference_table_level: int | None
    scaling_code: str
    displacement_code: str
    table_level_code: str
    notes: str


class NearFieldEvalBase:
    """Base class of near-field evaluators (``list1.py:83-215``)."""

    default_name = "near_field_eval_base"

    def _supports_inferred_scaling(self):
        return False

    def __init__(self, integral_kernel, table_data_shapes, potential_kind=1,
                 options=None, name=None, device=None, **kwargs):
        if options is None:
            options = []
        self.integral_kernel = integral_kernel
        self.n_tables = table_data_shapes["n_tables"]
        self.n_q_points = table_data_shapes["n_q_points"]
        self.n_table_entries = table_data_shapes["n_table_entries"]
        self.n_cases = table_data_shapes.get("n_cases", 0)
        self.reconstruction_kind = table_data_shapes.get("reconstruction_kind", "dense")
        self.n_arithmetic_case_orbits = table_data_shapes.get("n_arithmetic_case_orbits", 0)
        self.potential_kind = potential_kind
        for v in (self.n_tables, self.n_q_points, self.n_table_entries, self.n_cases):
            assert np.isreal(v)
        assert self.reconstruction_kind in {
            "dense", "generated-orbit", "scalar-arithmetic-orbit",
            "signed-arithmetic-orbit"}
        self.options = options
        self.name = name or self.default_name
        self.device = device
        self.extra_kwargs = kwargs
        self.kname = repr(self.integral_kernel)
        self.dim = self.integral_kernel.dim
        self.quad_order = int(table_data_shapes.get(
            "quad_order", round(float(self.n_q_points) ** (1.0 / float(self.dim)))))

        if "case_encoding_bias" not in self.extra_kwargs:
            self.extra_kwargs["case_encoding_bias"] = CASE_ENCODING_BIAS_DEFAULT
        self.extra_kwargs["case_encoding_bias"] = float(self.extra_kwargs["case_encoding_bias"])
        if self.extra_kwargs.get("case_encoding_warn_tol") is not None:
            self.extra_kwargs["case_encoding_warn_tol"] = float(
                self.extra_kwargs["case_encoding_warn_tol"])

        if "infer_kernel_scaling" not in self.extra_kwargs:
            self.extra_kwargs["infer_kernel_scaling"] = (
                self.n_tables == 1 and self._supports_inferred_scaling())

        if (self.extra_kwargs.get("infer_kernel_scaling", False)
                and not self._supports_inferred_scaling()
                and "kernel_scaling_code" not in self.extra_kwargs):
            raise RuntimeError(
                "infer_kernel_scaling is unsupported for kernel "
                f"{self.integral_kernel!r}. For Helmholtz, "
                "K_k(h r) = h^{-1} K_{k h}(r): exact table scaling requires "
                "changing the effective wave number with box size, which a "
                "single fixed-k table cannot represent. Use multi-level tables "
                "or provide explicit custom scaling/displacement code.")

        if ("kernel_scaling_code" in self.extra_kwargs
                or "kernel_displacement_code" in self.extra_kwargs):
            self.extra_kwargs["infer_kernel_scaling"] = False
            assert ("kernel_scaling_code" in self.extra_kwargs
                    and "kernel_displacement_code" in self.extra_kwargs)

        self._single_table_level_check_cache_key = None

    def get_cache_key(self):
        return (type(self).__name__, self.name, self.kname,
                "infer_scaling=" + str(self.extra_kwargs["infer_kernel_scaling"]))


# {{{ policy string -> kernel parameters

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _strip(code):
    return re.sub(r"[\s\\]+", "", str(code))


def _split_top_level_div(expr):
    depth = 0
    for i, ch in enumerate(expr):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "/" and depth == 0:
            return expr[:i], expr[i + 1:]
    return expr, None


def _factor_count(expr, box_name):
    """Count factors of a product of ``box_extent`` / ``table_root_extent``."""
    e = expr
    while e.startswith("(") and e.endswith(")"):
        e = e[1:-1]
    if e in ("1", "1.0"):
        return 0, 0
    n_box = n_tab = 0
    for f in e.split("*"):
        if f == f"{box_name}_extent":
            n_box += 1
        elif f == "table_root_extent":
            n_tab += 1
        else:
            raise NotImplementedError(f"unsupported factor {f!r} in a scaling code")
    return n_box, n_tab


def parse_scaling_code(code, box_name="sbox"):
    """Exponent p of ``scaling = (box_extent / table_root_extent)**p``."""
    s = _strip(code)
    if s in ("1.0", "1", "(1.0)"):
        return 0
    num, den = _split_top_level_div(s)
    if den is None:
        raise NotImplementedError(f"unsupported scaling code {code!r}")
    nb, nt = _factor_count(num, box_name)
    db, dt = _factor_count(den, box_name)
    if nb and not nt and dt == nb and not db:
        return nb
    if nt and not nb and db == nt and not dt:
        return -nt
    raise NotImplementedError(f"unsupported scaling code {code!r}")


def parse_displacement_code(code, box_name="sbox"):
    """``(kind, coef)``: ``0.0`` or ``a / b * scaling * log(box/table) * mode_nmlz``."""
    s = _strip(code)
    if s in ("0.0", "0", "(0.0)"):
        return _lib.VL1_DISP_NONE, 0.0
    m = re.fullmatch(
        rf"(?P<neg>-?)(?P<a>{_NUM})/\(?(?P<b>{_NUM})\)?\*scaling\*"
        rf"log\({box_name}_extent/table_root_extent\)\*mode_nmlz\[table_lev,sid\]", s)
    if m is None:
        raise NotImplementedError(f"unsupported displacement code {code!r}")
    coef = float(m.group("a")) / float(m.group("b"))
    if m.group("neg"):
        coef = -coef
    return _lib.VL1_DISP_LOG2D, coef


def parse_table_level_code(code, box_name="sbox"):
    s = _strip(code)
    if s in ("0.0", "0"):
        return _lib.VL1_LEVEL_ZERO
    per_level = _strip(
        f"(0 if {box_name}_level < table_starting_level "
        f"else ({box_name}_level - table_starting_level "
        f"if {box_name}_level - table_starting_level < n_tables "
        "else n_tables - 1))")
    if s == per_level:
        return _lib.VL1_LEVEL_PER_LEVEL
    raise NotImplementedError(f"unsupported table level code {code!r}")


def parse_policy(policy: KernelScalingPolicy):
    """Kernel parameters of a :class:`KernelScalingPolicy`."""
    p = parse_scaling_code(policy.scaling_code)
    disp_kind, disp_coef = parse_displacement_code(policy.displacement_code)
    level = parse_table_level_code(policy.table_level_code)
    return {"scaling_exponent": p, "displacement_kind": disp_kind,
            "displacement_coef": disp_coef, "table_level_kind": level}

# }}}


def _array_token(ary):
    if hasattr(ary, "data_ptr"):
        return ("t", int(ary.data_ptr()), int(getattr(ary, "_version", 0)),
                tuple(ary.shape), str(ary.dtype))
    if isinstance(ary, np.ndarray):
        return ("np", int(ary.ctypes.data), tuple(ary.shape), ary.dtype.str)
    return ("py", id(ary))


def _to_numpy(x):
    if x is None:
        return None
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    if hasattr(x, "get"):
        return np.asarray(x.get())
    return np.asarray(x)


class NearFieldFromCSR(NearFieldEvalBase):
    """Evaluate the near-field potentials from CSR representation of the tree.
    The class supports auto-scaling of simple kernels."""

    default_name = "near_field_from_csr"

    # {{{ kernel classification (list1.py:230-276)

    def _base_kernel(self):
        return base_kernel(self.integral_kernel)

    def _is_laplace_kernel(self, dim):
        return kernel_class_name(self._base_kernel()) == "LaplaceKernel" and self.dim == dim

    def _is_constant_kernel(self, dim):
        return self.kname in {f"CstKnl{dim}D", f"ConstantKernel{dim}D"} or (
            kernel_class_name(self._base_kernel()) == "ConstantKernel" and self.dim == dim)

    def _is_axis_derivative_of_laplace(self, cls, dim):
        k = self.integral_kernel
        return (kernel_class_name(k) == cls
                and kernel_class_name(base_kernel(k.inner_kernel)) == "LaplaceKernel"
                and self.dim == dim)

    def _is_axis_target_derivative_of_laplace(self, dim):
        return self._is_axis_derivative_of_laplace("AxisTargetDerivative", dim)

    def _is_axis_source_derivative_of_laplace(self, dim):
        return self._is_axis_derivative_of_laplace("AxisSourceDerivative", dim)

    def _supports_inferred_scaling(self):
        return any(f(d) for d in (2, 3) for f in (
            self._is_laplace_kernel, self._is_constant_kernel,
            self._is_axis_target_derivative_of_laplace,
            self._is_axis_source_derivative_of_laplace))

    # }}}

    # {{{ policy strings (list1.py:278-437)

    def _inferred_scaling_code(self):
        if any(f(d) for d in (2, 3) for f in (self._is_axis_target_derivative_of_laplace,
                                              self._is_axis_source_derivative_of_laplace)):
            return "BOX_extent / table_root_extent"
        if self._is_laplace_kernel(2) or self._is_constant_kernel(2) or \
                self._is_laplace_kernel(3):
            return "BOX_extent * BOX_extent / \
                    (table_root_extent * table_root_extent)"
        if self._is_constant_kernel(3):
            return "BOX_extent * BOX_extent * BOX_extent / \
                    (table_root_extent * table_root_extent * table_root_extent)"
        raise RuntimeError(f"no inferred scaling rule for {self.integral_kernel!r}")

    def _inferred_displacement_code(self):
        if any(f(d) for d in (2, 3) for f in (self._is_axis_target_derivative_of_laplace,
                                              self._is_axis_source_derivative_of_laplace)):
            return "0.0"
        if self._is_laplace_kernel(2):
            s = "-0.5 / PI * scaling * \
                    log(BOX_extent / table_root_extent) * \
                    mode_nmlz[table_lev, sid]"
            return s.replace("PI", str(math.pi))
        if self._supports_inferred_scaling():
            return "0.0"
        raise RuntimeError(f"no inferred displacement rule for {self.integral_kernel!r}")

    def _inferred_table_level_code(self):
        return "0.0"

    def get_kernel_scaling_policy(self, box_name="sbox"):
        """Return the table-level and scaling policy (``list1.py:361-437``).

        ``canonical_single_table``: table level 0 for all source-box levels with
        inferred scaling/displacement; ``custom_single_table``: user codes;
        ``fixed_single_table``: the one table without scaling (source levels
        must match the table level); ``per_level_tables``: one table per
        source-box level, no scaling.
        """
        if self.extra_kwargs.get("infer_kernel_scaling", False):
            return KernelScalingPolicy(
                kernel_name=self.kname, mode="canonical_single_table",
                infer_kernel_scaling=True, single_table_scaling_supported=True,
                reference_table_level=0,
                scaling_code=self._inferred_scaling_code().replace("BOX", box_name),
                displacement_code=self._inferred_displacement_code().replace("BOX", box_name),
                table_level_code=self._inferred_table_level_code().replace("BOX", box_name),
                notes="Uses table level 0 for all source-box levels with inferred exact scaling.")
        if "kernel_scaling_code" in self.extra_kwargs:
            return KernelScalingPolicy(
                kernel_name=self.kname, mode="custom_single_table",
                infer_kernel_scaling=False, single_table_scaling_supported=True,
                reference_table_level=0,
                scaling_code=self.extra_kwargs["kernel_scaling_code"].replace("BOX", box_name),
                displacement_code=self.extra_kwargs["kernel_displacement_code"].replace(
                    "BOX", box_name),
                table_level_code="0.0",
                notes="Uses user-provided scaling and displacement code with table level 0.")
        if self.n_tables == 1:
            return KernelScalingPolicy(
                kernel_name=self.kname, mode="fixed_single_table",
                infer_kernel_scaling=False, single_table_scaling_supported=False,
                reference_table_level=0, scaling_code="1.0", displacement_code="0.0",
                table_level_code="0.0",
                notes=("Uses the only cached table level without kernel scaling; "
                       "runtime checks reject mixed source levels or a table level mismatch."))
        return KernelScalingPolicy(
            kernel_name=self.kname, mode="per_level_tables", infer_kernel_scaling=False,
            single_table_scaling_supported=False, reference_table_level=None,
            scaling_code="1.0", displacement_code="0.0",
            table_level_code=(
                "(0 if BOX_level < table_starting_level "
                "else (BOX_level - table_starting_level "
                "if BOX_level - table_starting_level < n_tables "
                "else n_tables - 1))").replace("BOX", box_name),
            notes="Selects one cached table level per source-box level without kernel scaling.")

    def codegen_compute_scaling(self, box_name="sbox"):
        return self.get_kernel_scaling_policy(box_name=box_name).scaling_code

    def codegen_compute_displacement(self, box_name="sbox"):
        return self.get_kernel_scaling_policy(box_name=box_name).displacement_code

    def codegen_get_table_level(self, box_name="sbox"):
        return self.get_kernel_scaling_policy(box_name=box_name).table_level_code

    def codegen_vec_component(self, d=None):
        dimension = self.dim - 1 if d is None else d
        bias = float(self.extra_kwargs["case_encoding_bias"])
        return ("((box_centers[" + str(dimension) + ", target_box_id]"
                "- box_centers[" + str(dimension) + ", source_box_id]"
                ") / sbox_extent * 4.0 + encoding_shift" + f" + {bias:.17g}" + ")")

    def codegen_vec_id(self):
        code = "0.0"
        for d in range(self.dim):
            code = "(" + code + ") * encoding_base"
            code = code + "+" + self.codegen_vec_component(d)
        return code

    def codegen_exterior_part(self):
        if self.potential_kind == 1:
            return "0.0"
        if self.potential_kind == 2:
            return "source_coefs[target_id] * ext_nmlz"
        raise ValueError("Unsupported potential kind %d" % self.potential_kind)

    def _target_batch_size(self):
        n = int(self.extra_kwargs.get("list1_target_batch_size", 1))
        if n < 1:
            raise ValueError("list1_target_batch_size must be positive")
        return n

    def get_cache_key(self):
        return (type(self).__name__, "vl1-gb300", self.name, self.kname,
                "complex_kernel=" + str(self.integral_kernel.is_complex_valued),
                "potential_kind=%d" % self.potential_kind,
                "reconstruction_kind=" + self.reconstruction_kind,
                "n_arithmetic_case_orbits=%d" % self.n_arithmetic_case_orbits,
                "infer_scaling=" + str(self.extra_kwargs["infer_kernel_scaling"]),
                "case_encoding_bias=" + repr(self.extra_kwargs["case_encoding_bias"]),
                "scaling_policy=" + self.codegen_compute_scaling(),
                "displacement_policy=" + self.codegen_compute_displacement(),
                "table_level_policy=" + self.codegen_get_table_level())

    # }}}

    # {{{ host checks the reference performs (list1.py:468-530, 1356-1399)

    def _warn_case_encoding_drift(self, box_centers, box_levels, root_extent,
                                  target_boxes, starts, lists, encoding_shift, warn_tol):
        if warn_tol is None:
            return
        bc = _to_numpy(box_centers)
        bl = _to_numpy(box_levels).astype(np.int64)
        tb = _to_numpy(target_boxes).astype(np.int64)
        st = _to_numpy(starts).astype(np.int64)
        ls = _to_numpy(lists).astype(np.int64)
        if tb.size == 0 or ls.size == 0:
            return
        tgt = np.repeat(tb, np.diff(st))
        ext = float(root_extent) * 0.5 ** bl[ls]
        raw = (bc[:, tgt] - bc[:, ls]) / ext[None, :] * 4.0 + float(encoding_shift)
        drift = np.abs(raw - np.rint(raw))
        k = int(np.argmax(drift))
        d, j = np.unravel_index(k, drift.shape)
        if drift.flat[k] > warn_tol:
            logger.warning(
                "List1 case encoding drift %.3e exceeds %.3e for target box %d, "
                "source box %d, dim %d (raw %.17g)", drift.flat[k], warn_tol,
                int(tgt[j]), int(ls[j]), int(d), float(raw[d, j]))

    def _check_single_table_levels(self, lists, box_levels, table_starting_level):
        if not (self.n_tables == 1
                and not self.extra_kwargs.get("infer_kernel_scaling", False)
                and "kernel_scaling_code" not in self.extra_kwargs):
            return
        key = (_array_token(lists), _array_token(box_levels), int(table_starting_level))
        if key == self._single_table_level_check_cache_key:
            return
        src = _to_numpy(lists)
        if src.size:
            lev = _to_numpy(box_levels)[src.astype(np.int64)]
            lo, hi = int(lev.min()), int(lev.max())
            if lo != hi:
                raise RuntimeError(
                    "Single near-field table without scaling cannot be used "
                    f"with source boxes on multiple levels ({lo}..{hi}); build per-level "
                    "tables or provide explicit scaling rules.")
            if lo != int(table_starting_level):
                raise RuntimeError(
                    "Single near-field table level mismatch: source level "
                    f"{lo} but table_starting_level is {int(table_starting_level)}. "
                    "Build the table at the active source level or provide scaling rules.")
        self._single_table_level_check_cache_key = key

    # }}}

    def _reconstruction_code(self):
        if self.reconstruction_kind == "scalar-arithmetic-orbit":
            return _lib.VL1_RECON_SCALAR_ARITH
        if self.reconstruction_kind == "signed-arithmetic-orbit":
            return _lib.VL1_RECON_SIGNED_ARITH
        if self.reconstruction_kind == "dense":
            return _lib.VL1_RECON_DENSE
        raise NotImplementedError(
            f"reconstruction kind {self.reconstruction_kind!r} has no GB300 kernel; "
            "the arithmetic orbit reconstruction (scalar/signed) and the dense table "
            "are supported")

    def _policy_and_key(self):
        """(parsed policy, cache key), recomputed only when ``extra_kwargs``
        changes (both derive from the kernel, fixed at construction, and the
        extra keyword arguments).  Scalars (numpy scalars included) enter the
        memo key by value, lists, tuples and dicts by their ``repr`` (so that
        changes made in place are seen), other objects by identity; the memo
        holds those objects, so that an identity cannot be reused while the
        memo stands."""
        snap = tuple(sorted((k, _memo_token(v)) for k, v in self.extra_kwargs.items()))
        memo = getattr(self, "_policy_memo", None)
        if memo is None or memo[0] != snap:
            held = [v for v in self.extra_kwargs.values() if not _is_scalar(v)]
            memo = (snap, parse_policy(self.get_kernel_scaling_policy()), self.get_cache_key(),
                    held)
            self._policy_memo = memo
        return memo[1], memo[2]

    def get_plan(self, *, table_data_combined, mode_nmlz_combined, case_indices,
                 encoding_base, encoding_shift, table_root_extent, table_starting_level,
                 arithmetic_case_orbit_ranks, arithmetic_case_axis_perm,
                 arithmetic_case_axis_sign, arithmetic_case_axis_group,
                 arithmetic_case_value_offsets, arithmetic_axis_sign_power,
                 arithmetic_axis_direction_signs, arithmetic_direction_sign_axis,
                 cache=True):
        """The device plan of this table payload (cached per payload identity;
        ``cache=False``: a new plan owned by the caller)."""
        from .plan import Plan, plan_cache_get
        policy, cache_key = self._policy_and_key()
        key = (cache_key, _array_token(table_data_combined),
               _array_token(mode_nmlz_combined), _array_token(case_indices),
               _array_token(arithmetic_case_orbit_ranks), _array_token(arithmetic_case_axis_perm),
               _array_token(arithmetic_case_axis_sign), _array_token(arithmetic_case_axis_group),
               _array_token(arithmetic_case_value_offsets), int(encoding_base),
               float(encoding_shift), float(table_root_extent), int(table_starting_level),
               int(arithmetic_direction_sign_axis))
        get = plan_cache_get if cache else (lambda _key, **kw: Plan(**kw))
        return get(
            key, dim=self.dim, quad_order=self.quad_order, n_tables=self.n_tables,
            table_data=_to_numpy(table_data_combined), mode_nmlz=_to_numpy(mode_nmlz_combined),
            case_indices=_to_numpy(case_indices), encoding_base=int(encoding_base),
            encoding_shift=float(encoding_shift),
            case_encoding_bias=float(self.extra_kwargs["case_encoding_bias"]),
            case_orbit_ranks=_to_numpy(arithmetic_case_orbit_ranks),
            case_axis_perm=_to_numpy(arithmetic_case_axis_perm),
            case_axis_sign=_to_numpy(arithmetic_case_axis_sign),
            case_axis_group=_to_numpy(arithmetic_case_axis_group),
            case_value_offsets=_to_numpy(arithmetic_case_value_offsets),
            axis_sign_power=_to_numpy(arithmetic_axis_sign_power),
            axis_direction_signs=_to_numpy(arithmetic_axis_direction_signs),
            direction_sign_axis=int(arithmetic_direction_sign_axis),
            reconstruction_kind=self._reconstruction_code(),
            table_root_extent=float(table_root_extent),
            table_starting_level=int(table_starting_level), **policy)

    def __call__(self, queue=None, **kwargs):
        """Evaluate list 1 into ``result`` (``list1.py:1260-1487``).

        Takes the reference's keyword arguments.  Returns ``(result, event)``.
        Extra keyword ``sync`` (default True, as the reference finishes the
        queue) reads the device status word and raises on invalid input.
        """
        import torch

        from .plan import as_device_tensor, stream_handle, tree_view_from_arrays
        if self.potential_kind != 1:
            raise NotImplementedError(
                "potential_kind=2 (hypersingular exterior part) is not implemented "
                "on GB300")
        self._target_batch_size()
        sync = kwargs.pop("sync", True)

        result = kwargs.pop("result")
        box_centers = kwargs.pop("box_centers")
        box_levels = kwargs.pop("box_levels")
        box_source_counts_nonchild = kwargs.pop("box_source_counts_nonchild")
        box_source_starts = kwargs.pop("box_source_starts")
        box_target_counts_nonchild = kwargs.pop("box_target_counts_nonchild")
        box_target_starts = kwargs.pop("box_target_starts")
        case_indices = kwargs.pop("case_indices")
        encoding_base = kwargs.pop("encoding_base")
        encoding_shift = kwargs.pop("encoding_shift")
        mode_nmlz_combined = kwargs.pop("mode_nmlz_combined")
        kwargs.pop("exterior_mode_nmlz_combined", None)
        recon = {k: kwargs.pop(k) for k in (
            "arithmetic_case_orbit_ranks", "arithmetic_case_axis_perm",
            "arithmetic_case_axis_sign", "arithmetic_case_axis_group",
            "arithmetic_case_value_offsets", "arithmetic_axis_sign_power",
            "arithmetic_axis_direction_signs", "arithmetic_direction_sign_axis")
            if k in kwargs}
        self._reconstruction_code()
        root_extent = kwargs.pop("root_extent")
        table_root_extent = kwargs.pop("table_root_extent")
        table_starting_level = kwargs.pop("table_starting_level")
        starts = kwargs.pop("neighbor_source_boxes_starts")
        lists = kwargs.pop("neighbor_source_boxes_lists")
        mode_coefs = kwargs.pop("mode_coefs")
        table_data_combined = kwargs.pop("table_data_combined")
        target_boxes = kwargs.pop("target_boxes")
        source_mode_ids = kwargs.pop("source_mode_ids")
        target_point_ids = kwargs.pop("target_point_ids")

        self._check_single_table_levels(lists, box_levels, table_starting_level)
        self._warn_case_encoding_drift(box_centers, box_levels, root_extent, target_boxes,
                                       starts, lists, encoding_shift,
                                       self.extra_kwargs.get("case_encoding_warn_tol"))

        plan = self.get_plan(
            table_data_combined=table_data_combined, mode_nmlz_combined=mode_nmlz_combined,
            case_indices=case_indices, encoding_base=encoding_base,
            encoding_shift=encoding_shift, table_root_extent=table_root_extent,
            table_starting_level=table_starting_level, **recon)

        view, keep = tree_view_from_arrays(
            target_boxes=target_boxes, neighbor_source_boxes_starts=starts,
            neighbor_source_boxes_lists=lists, box_centers=box_centers,
            box_levels=box_levels, box_source_starts=box_source_starts,
            box_source_counts_nonchild=box_source_counts_nonchild,
            box_target_starts=box_target_starts,
            box_target_counts_nonchild=box_target_counts_nonchild,
            source_mode_ids=source_mode_ids, target_point_ids=target_point_ids,
            root_extent=root_extent)

        coefs = as_device_tensor(mode_coefs)
        if coefs.dtype not in (torch.float64, torch.complex128):
            coefs = coefs.to(torch.complex128 if coefs.is_complex() else torch.float64)
        out_complex = plan.complex_table or coefs.is_complex()
        out_dtype = torch.complex128 if out_complex else torch.float64

        np_result = None
        if isinstance(result, np.ndarray) or not (hasattr(result, "is_cuda") and result.is_cuda):
            np_result = result
            out = torch.empty(int(view.n_particles), dtype=out_dtype, device="cuda")
        else:
            out = result
            if out.dtype != out_dtype or not out.is_contiguous():
                raise ValueError(
                    f"result must be a contiguous {out_dtype} CUDA tensor, got "
                    f"{out.dtype}")

        stream = stream_handle(queue)
        precision = self.extra_kwargs.get("list1_precision", "fp64")
        if precision == "fp64":
            plan.eval_fp64(view, coefs, out, stream=stream, nrhs=1)
        elif precision == "mixed":
            from .batched import eval_mixed
            eval_mixed(plan, view, coefs, out, stream=stream, nrhs=1, keep=keep)
        else:
            raise ValueError(f"list1_precision must be 'fp64' or 'mixed', got {precision!r}")
        evt = torch.cuda.Event()
        evt.record(torch.cuda.current_stream() if queue is None else queue)
        del keep
        if sync:
            plan.raise_on_status(stream)
        if np_result is not None:
            host = out.cpu().numpy()
            if isinstance(np_result, np.ndarray) and np_result.shape == host.shape:
                np_result[...] = host
                return np_result, evt
            return host, evt
        return out, evt
