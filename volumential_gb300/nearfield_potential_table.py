"""Near-field interaction table: data model of the list-1 path.

Mirrors the attributes and methods of ``NearFieldInteractionTable``
(``volumential/nearfield_potential_table.py:436-1249``) that the list-1 path
reads: the quadrature-point layout, the case gallery, entry-id conventions,
the compact (orbit-reduced) storage and the arithmetic orbit metadata.

Conventions (reference line numbers):

* source box is ``[0, source_box_extent]^dim``; ``q_points`` are the tensor
  Gauss-Legendre nodes mapped to it, lexicographic with axis 0 slowest
  (``:565-592``);
* full entry id ``case * n_pairs + source_mode * n_q_points + target_point``
  (``:653-664``, inverse ``:670-685``);
* 2D ``mode_normalizers`` are the outer product of the mapped Gauss-Legendre
  weights (``:2744-2770``), 3D normalizers stay zero (``:539``);
* a compact table stores one value per orbit representative, addressed by
  ``reduced_entry_ids`` (``:1015-1083``).

Table VALUES come from a builder: the constant kernel has a closed form (the
mapped Gauss-Legendre weight of the source mode); other kernels are filled by
``set_reduced_table_data`` from a table builder or from stored data.
"""

from __future__ import annotations

import numpy as np

from . import list1_gallery as gallery
from .orbit_arithmetic import (
    build_arithmetic_case_metadata,
    decode_mode_axes,
    enumerate_scalar_arithmetic_representatives,
)

__all__ = ["NearFieldInteractionTable", "constant_one"]


def constant_one(*args):
    return 1.0


_INVARIANT_CACHE: dict = {}


class NearFieldInteractionTable:
    """Precomputed singular integrals of one kernel on template boxes."""

    def __init__(self, quad_order, method="gauss-legendre", dim=2, kernel_func=None,
                 kernel_type=None, sumpy_kernel=None, build_method="DuffyRadial",
                 source_box_extent=1, dtype=np.float64, derive_kernel_func=True,
                 progress_bar=False, **kwargs):
        if dim not in (1, 2, 3):
            raise NotImplementedError
        if source_box_extent <= 0:
            raise ValueError("source_box_extent must be positive")
        if method != "gauss-legendre" and kwargs.get("precomputed_q_points") is None:
            raise NotImplementedError(method)
        self.quad_order = int(quad_order)
        self.dim = int(dim)
        self.dtype = np.dtype(dtype).type
        self.source_box_extent = float(source_box_extent)
        self.center = np.full(self.dim, 0.5 * self.source_box_extent)
        self.build_method = build_method
        self.kernel_func = kernel_func
        if sumpy_kernel is None and kernel_func is None and dim == 2:
            kernel_type = "const"
        self.kernel_type = kernel_type
        self.integral_knl = sumpy_kernel
        self.symmetry_source_direction = kwargs.pop("symmetry_source_direction", None)

        self.n_q_points = self.quad_order ** self.dim
        self.n_pairs = self.n_q_points ** 2
        self.mode_normalizers = np.zeros(self.n_q_points, dtype=self.dtype)
        self.kernel_exterior_normalizers = np.zeros(self.n_q_points, dtype=self.dtype)

        self.interaction_case_vecs, self.case_encode, self.case_indices = \
            gallery.generate_list1_gallery(self.dim)
        self.n_cases = len(self.interaction_case_vecs)

        pre = kwargs.pop("precomputed_q_points", None)
        if pre is not None:
            pre = np.asarray(pre, dtype=np.float64)
            if pre.shape != (self.n_q_points, self.dim):
                raise ValueError(
                    f"precomputed_q_points has shape {pre.shape}, expected "
                    f"{(self.n_q_points, self.dim)}")
            self.q_points = pre
        else:
            x, _ = np.polynomial.legendre.leggauss(self.quad_order)
            nodes = 0.5 * self.source_box_extent * (x + 1.0)
            grids = np.meshgrid(*([nodes] * self.dim), indexing="ij")
            self.q_points = np.stack([g.ravel() for g in grids], axis=1)

        self.reduced_entry_ids = None
        self._data = None
        self.table_data_is_symmetry_reduced = False
        self.is_built = False
        self.build_extra_kwargs = kwargs

    # {{{ storage

    def _full_entry_count(self):
        return self.n_cases * self.n_pairs

    @property
    def data(self):
        if self._data is None:
            self._data = np.full(self._full_entry_count(), np.nan, dtype=self.dtype)
        return self._data

    @data.setter
    def data(self, value):
        self._data = np.asarray(value, dtype=self.dtype)
        self.reduced_entry_ids = None
        self.table_data_is_symmetry_reduced = False

    def get_entry_index(self, source_mode_index, target_point_index, case_id):
        assert 0 <= source_mode_index < self.n_q_points
        assert 0 <= target_point_index < self.n_q_points
        return int(case_id * self.n_pairs + source_mode_index * self.n_q_points
                   + target_point_index)

    def decode_index(self, entry_id):
        case_id, pair_id = divmod(int(entry_id), self.n_pairs)
        s, t = divmod(pair_id, self.n_q_points)
        return {"case_index": case_id, "source_mode_index": s, "target_point_index": t}

    def unwrap_mode_index(self, mode_index):
        return decode_mode_axes(mode_index, self.quad_order, self.dim)

    def get_reduced_entry_ids(self):
        if not self.table_data_is_symmetry_reduced:
            if self._data is None:
                return np.empty(0, dtype=np.int64)
            return np.arange(len(self._data), dtype=np.int64)
        return np.asarray(self.reduced_entry_ids, dtype=np.int64)

    def get_reduced_table_data(self):
        """``(full_entry_ids, values)`` of the stored entries."""
        if self._data is None:
            return np.empty(0, dtype=np.int64), np.empty(0, dtype=self.dtype)
        return self.get_reduced_entry_ids(), np.asarray(self._data)

    def set_reduced_table_data(self, entry_ids, values):
        """Store values compactly by full entry id (sorted, unique)."""
        entry_ids = np.asarray(entry_ids, dtype=np.int64)
        values = np.asarray(values, dtype=self.dtype)
        if entry_ids.ndim != 1 or values.ndim != 1:
            raise ValueError("entry_ids and values must be one-dimensional")
        if entry_ids.shape != values.shape:
            raise ValueError(
                "entry_ids and values must have the same shape for reduced storage")
        order = np.argsort(entry_ids, kind="stable")
        entry_ids, values = entry_ids[order], values[order]
        if entry_ids.size:
            if entry_ids[0] < 0 or entry_ids[-1] >= self._full_entry_count():
                raise ValueError("entry_ids must be valid full table entry IDs")
            if np.any(entry_ids[1:] == entry_ids[:-1]):
                raise ValueError("entry_ids must be unique")
        self.reduced_entry_ids = np.ascontiguousarray(entry_ids)
        self._data = np.ascontiguousarray(values)
        self.table_data_is_symmetry_reduced = True
        self.is_built = True

    def get_entry_data_for_full_indices(self, entry_ids):
        entry_ids = np.asarray(entry_ids, dtype=np.int64)
        if not self.table_data_is_symmetry_reduced:
            if self._data is None:
                raise RuntimeError("table data has not been built")
            return np.asarray(self._data)[entry_ids]
        stored = self.get_reduced_entry_ids()
        pos = np.searchsorted(stored, entry_ids)
        if np.any(pos >= len(stored)) or not np.array_equal(stored[np.minimum(
                pos, len(stored) - 1)], entry_ids):
            raise RuntimeError(
                "missing canonical table entry data for compact orbit-reduced table")
        return np.asarray(self._data)[pos]

    def has_entry_data_for_full_indices(self, entry_ids):
        try:
            vals = self.get_entry_data_for_full_indices(entry_ids)
        except RuntimeError:
            return False
        return bool(np.all(np.isfinite(vals)))

    # }}}

    # {{{ orbit metadata (volumential/nearfield_potential_table.py:1200-1249)

    def _orbit_cache_key(self):
        return (self.dim, self.quad_order, repr(self.integral_knl))

    def _get_scalar_arithmetic_invariant_entry_info(self):
        """Orbit representatives and arithmetic metadata: the scalar symmetry,
        or for derivative kernels the signed one (differentiated axes fixed
        and odd); ``None`` (full table, dense reconstruction) for kernels
        without an arithmetic symmetry."""
        from .kernels import arithmetic_symmetry

        if self.dim not in (2, 3):
            return None
        sym = (None if self.integral_knl is None
               else arithmetic_symmetry(self.integral_knl, self.dim))
        if sym is False:
            return None   # full table, dense reconstruction
        sym_key = None if sym is None else (
            tuple(sym["axis_groups"]), tuple(int(v) for v in sym["axis_sign_power"]))
        key = ("arithmetic", self.dim, self.quad_order, sym_key)
        hit = _INVARIANT_CACHE.get(key)
        if hit is not None:
            return hit
        md = build_arithmetic_case_metadata(self, sym)
        if md is None:
            return None
        entry_ids = enumerate_scalar_arithmetic_representatives(self, md)
        info = {
            "kind": "scalar-arithmetic-orbit" if sym is None else "signed-arithmetic-orbit",
            "entry_ids": entry_ids,
            "case_indices": (entry_ids // self.n_pairs).astype(np.int32),
            "source_mode_indices": ((entry_ids % self.n_pairs)
                                    // self.n_q_points).astype(np.int32),
            "target_point_indices": (entry_ids % self.n_q_points).astype(np.int32),
            "arithmetic_metadata": {k: v for k, v in md.items()
                                    if k != "case_value_offsets_i64"},
        }
        _INVARIANT_CACHE[key] = info
        return info

    def _get_invariant_entry_info(self):
        return self._get_scalar_arithmetic_invariant_entry_info()

    # }}}

    # {{{ geometry of the cases (volumential/nearfield_potential_table.py:917-946)

    def case_target_box(self, case_index):
        """Centre and relative size of the target box of a case."""
        vec = np.asarray(self.interaction_case_vecs[case_index], dtype=np.float64)
        center = self.center + vec / 4.0 * self.source_box_extent
        m = int(np.max(np.abs(vec)))
        size = 1.0 if m == 0 else (m - 2.0) / 2.0
        return center, size

    def find_target_point(self, target_point_index, case_index):
        center, size = self.case_target_box(case_index)
        return center + size * (self.q_points[target_point_index] - self.center)

    def get_case_target_points(self):
        """Target points of every case: ``[dim, n_cases, n_q_points]``."""
        out = np.empty((self.dim, self.n_cases, self.n_q_points))
        for c in range(self.n_cases):
            center, size = self.case_target_box(c)
            out[:, c, :] = (center[:, None]
                            + size * (self.q_points - self.center).T)
        return out

    # }}}

    # {{{ builders

    def build_normalizer_table(self, pool=None, pb=None):
        """2D: outer product of the mapped Gauss-Legendre weights."""
        if self.dim != 2:
            raise NotImplementedError("normalizers are defined in 2D only")
        _, w = np.polynomial.legendre.leggauss(self.quad_order)
        w = 0.5 * self.source_box_extent * w
        self.mode_normalizers[:] = np.multiply.outer(w, w).reshape(-1)

    def mode_weights(self):
        """Integral of every source mode's Lagrange basis over the source box."""
        _, w = np.polynomial.legendre.leggauss(self.quad_order)
        w = 0.5 * self.source_box_extent * w
        out = w
        for _ in range(self.dim - 1):
            out = np.multiply.outer(out, w)
        return np.asarray(out).reshape(-1)

    def build_constant_table(self):
        """Exact table of the constant kernel K = 1: every entry is the integral
        of the source mode over the source box (its Gauss-Legendre weight)."""
        info = self._get_scalar_arithmetic_invariant_entry_info()
        ids = info["entry_ids"]
        smodes = info["source_mode_indices"]
        self.set_reduced_table_data(ids, self.mode_weights()[smodes].astype(self.dtype))
        if self.dim == 2:
            self.build_normalizer_table()

    def build_table_via_duffy_radial(self, radial_rule="tanh-sinh-fast",
                                     regular_quad_order=20, radial_quad_order=61,
                                     mp_dps=50, queue=None, cl_ctx=None, build_config=None,
                                     auto_tune_orders=False, auto_tune_samples=5,
                                     auto_tune_floor_factor=8.0, auto_tune_candidates=None,
                                     **kwargs):
        """Fill the table's orbit-invariant entries by Duffy radial quadrature
        in FP64 on the GPU (``nearfield_potential_table.py:2948-3195``; the
        fixed tanh-sinh rules of its batched path).  ``queue``: an optional
        ``torch.cuda.Stream``.  A Helmholtz kernel's wave number is passed by
        its argument name (``k`` by default).  ``max_ctas`` > 0 caps the
        builder's grid.  Orders ``"auto"`` / ``None``, ``auto_tune_orders``
        or a ``DuffyBuildConfig`` asking for it choose the orders by
        convergence on sample entries (``:2465-2619``; the choice is kept in
        ``last_duffy_order_selection``)."""
        from .plan import stream_handle
        from .table_builder import DuffyBuildConfig, autotune_duffy_orders, is_auto_order
        from .table_builder import build_table_values

        if build_config is None:
            build_config = DuffyBuildConfig(
                radial_rule=radial_rule, regular_quad_order=regular_quad_order,
                radial_quad_order=radial_quad_order, mp_dps=mp_dps,
                auto_tune_orders=auto_tune_orders, auto_tune_samples=auto_tune_samples,
                auto_tune_floor_factor=auto_tune_floor_factor,
                auto_tune_candidates=auto_tune_candidates)
        elif not isinstance(build_config, DuffyBuildConfig):
            raise TypeError("build_config must be a DuffyBuildConfig")
        base = self.integral_knl
        while hasattr(base, "inner_kernel"):
            base = base.inner_kernel
        name = getattr(base, "helmholtz_k_name", "k")
        k = kwargs.pop(name, kwargs.pop("k", None))
        kernel = kwargs.pop("kernel", None)
        max_ctas = int(kwargs.pop("max_ctas", 0))
        if kwargs:
            raise TypeError(f"unexpected keyword arguments {sorted(kwargs)}")
        sh = stream_handle(queue)
        reg, rad = build_config.regular_quad_order, build_config.radial_quad_order
        if (build_config.auto_tune_orders or is_auto_order(reg) or is_auto_order(rad)):
            reg, rad, info = autotune_duffy_orders(
                self, radial_rule=build_config.radial_rule, mp_dps=build_config.mp_dps,
                sample_count=build_config.auto_tune_samples,
                candidates=build_config.auto_tune_candidates,
                floor_factor=build_config.auto_tune_floor_factor, kernel=kernel, k=k,
                stream=sh)
            self.last_duffy_order_selection = info
        self.build_config = DuffyBuildConfig(
            radial_rule=build_config.radial_rule, regular_quad_order=int(reg),
            radial_quad_order=int(rad), mp_dps=build_config.mp_dps)
        build_table_values(self, radial_rule_name=build_config.radial_rule,
                           regular_quad_order=int(reg), radial_quad_order=int(rad),
                           mp_dps=build_config.mp_dps, kernel=kernel, k=k, stream=sh,
                           max_ctas=max_ctas)

    def build_table(self, cl_ctx=None, queue=None, build_config=None, **kwargs):
        """``nearfield_potential_table.py:3200``: the constant kernel's closed
        form, otherwise the Duffy radial builder."""
        name = type(self.integral_knl).__name__ if self.integral_knl is not None else None
        if self.kernel_type == "const" or name == "ConstantKernel":
            self.build_constant_table()
            return
        self.build_table_via_duffy_radial(queue=queue, build_config=build_config, **kwargs)

    # }}}
