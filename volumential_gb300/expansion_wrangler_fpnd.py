"""FPND expansion wrangler, list-1 stage ("Far field by Particles, Near field Direct").

Restates the list-1 part of ``volumential/expansion_wrangler_fpnd.py``:

* ``_compute_box_local_ids``               -- ``:408-424``
* ``_validate_table_box_particle_layout``  -- ``:427-514``
* ``_build_fast_scalar_arithmetic_orbit_reconstruction`` -- ``:1667-1726``
* ``_prepare_table_data_and_entry_map``    -- ``:1805-2066`` (arithmetic path)
* payload cache                            -- ``:2939-3158``
* ``eval_direct_single_out_kernel`` / ``eval_direct`` -- ``:3222-3489``

plus ``eval_direct_batched``: all right-hand sides of one call in one launch
(per-RHS outputs; ``drive_volume_fmm`` sums them, which is the reference's
superposition of fields, ``volume_fmm.py:1028-1031``).

The far-field stages of the reference's wrangler (multipoles, M2L, locals)
are not part of this package: the wrangler supports ``list1_only`` drives.
"""

from __future__ import annotations

import collections
import logging
import math

import numpy as np

from .expansion_wrangler_interface import ExpansionWranglerInterface
from .kernels import base_kernel
from .list1 import NearFieldFromCSR
from .orbit_arithmetic import metadata_nbytes

logger = logging.getLogger(__name__)

_ARITHMETIC_RECONSTRUCTION_KINDS = {"scalar-arithmetic-orbit", "signed-arithmetic-orbit"}

__all__ = [
    "FPNDExpansionWrangler", "FPNDSumpyExpansionWrangler",
    "FPNDTreeIndependentDataForWrangler", "_compute_box_local_ids",
    "_validate_table_box_particle_layout", "_prepare_table_data_and_entry_map",
    "_build_fast_scalar_arithmetic_orbit_reconstruction",
]


def _np(x):
    if x is None:
        return None
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    if hasattr(x, "get") and not isinstance(x, np.ndarray):
        return np.asarray(x.get())
    return np.asarray(x)


def _normalize_term_key(key):
    """A split term key as ("power" | "power_log", power): from a (kind,
    power) tuple, an int (a power of r) or a string "constant", "power:<n>",
    "power_log:<n>" (the accepted forms of expansion_wrangler_fpnd.py:
    335-376)."""
    if isinstance(key, tuple):
        if len(key) != 2:
            raise ValueError("helmholtz split term key tuples must have length 2: (kind, power)")
        kind, power = key
    elif isinstance(key, (int, np.integer)):
        kind, power = "power", key
    elif isinstance(key, str):
        if key == "constant":
            kind, power = "power", 0
        elif ":" in key and key.split(":", 1)[0] in ("power", "power_log"):
            kind, power = key.split(":", 1)
        else:
            raise ValueError("invalid helmholtz split term key string; expected one of: "
                             "constant, power:<n>, power_log:<n>")
    else:
        raise TypeError("helmholtz split term key must be int, str, or (kind, power) tuple")
    kind = str(kind)
    if kind not in ("power", "power_log"):
        raise ValueError("helmholtz split term key kind must be 'power' or 'power_log'")
    power = int(power)
    if power < 0:
        raise ValueError("helmholtz split term key power must be >= 0")
    if kind == "power_log" and power == 0:
        raise ValueError("helmholtz split power_log term requires power >= 1")
    return kind, power


def _compute_box_local_ids(tree, n_q_points):
    """Box-local particle index of every particle, in tree order."""
    if not getattr(tree, "sources_are_targets", False):
        raise ValueError(
            "table-based near-field evaluation requires sources and targets "
            "to coincide (tree.sources_are_targets=True)")
    n = int(tree.ntargets)
    if n % n_q_points != 0:
        raise ValueError("particle count is not divisible by box-local quadrature size")
    local = np.tile(np.arange(n_q_points, dtype=np.int32), n // n_q_points)
    return local[_np(tree.sorted_target_ids)]


def _validate_table_box_particle_layout(tree, target_boxes, source_boxes, n_q_points):
    counts = _np(tree.box_target_counts_nonchild)
    tc = counts[_np(target_boxes).astype(np.int64)]
    sc = counts[_np(source_boxes).astype(np.int64)]
    if np.all(tc == n_q_points) and np.all(sc == n_q_points):
        return
    bad_t = np.unique(tc[tc != n_q_points])
    bad_s = np.unique(sc[sc != n_q_points])
    raise ValueError(
        "table-based near-field evaluation requires exactly "
        f"{n_q_points} quadrature points per active source/target box; "
        f"found target counts {bad_t.tolist()} and source counts "
        f"{bad_s.tolist()}. Build the particle tree from the mesh box-tree "
        "(build_particle_tree_from_box_tree) to preserve per-cell quadrature layout.")


def _build_fast_scalar_arithmetic_orbit_reconstruction(table):
    if not hasattr(table, "_get_scalar_arithmetic_invariant_entry_info"):
        return None
    info = table._get_scalar_arithmetic_invariant_entry_info()
    if info is None:
        return None
    md = info["arithmetic_metadata"]
    layout = np.asarray(info["entry_ids"], dtype=np.int64)
    n_orbits = int(np.asarray(md["case_value_offsets"]).size - 1)
    return {
        "kind": info.get("kind", "scalar-arithmetic-orbit"),
        "case_orbit_ranks": np.asarray(md["case_orbit_ranks"], dtype=np.uint16),
        "case_axis_perm": np.asarray(md["case_axis_perm"], dtype=np.uint8),
        "case_axis_sign": np.asarray(md["case_axis_sign"], dtype=np.int8),
        "case_axis_group": np.asarray(md["case_axis_group"], dtype=np.uint8),
        "case_value_offsets": np.asarray(md["case_value_offsets"], dtype=np.int32),
        "axis_sign_power": np.asarray(md["axis_sign_power"], dtype=np.uint8),
        "axis_direction_signs": np.asarray(md["axis_direction_signs"], dtype=np.int8),
        "direction_sign_axis": int(md["direction_sign_axis"]),
        "layout_entry_ids": layout,
        "layout_entry_scales": np.ones(len(layout), dtype=np.int8),
        "n_case_orbits": n_orbits,
        "metadata_bytes": metadata_nbytes(md),
        "dense_arithmetic_layout_entry_count": int(n_orbits * table.n_pairs),
        "compact_value_entry_count": int(len(layout)),
        "representative_entry_count": int(len(layout)),
        "distinct_layout_entry_count": int(len(np.unique(layout))),
        "duplicate_layout_entry_count": 0,
        "unused_layout_entry_count": 0,
        "sign_convention_conflict_count": 0,
    }


def _prepare_table_data_and_entry_map(table_levels):
    """Compact table of every level, normalizers and the reconstruction info.

    Returns ``(table_data_combined, mode_nmlz_combined,
    exterior_mode_nmlz_combined, table_entry_ids, table_entry_scales,
    reconstruction_info)`` like the reference.  Reduced (orbit-compact) and
    full tables are both accepted; a full table contributes the values of the
    orbit representatives.  Kernels without an arithmetic orbit
    reconstruction (the reference's generated/dense fallbacks) raise.
    """
    if not table_levels:
        raise ValueError("table_levels cannot be empty")
    table0 = table_levels[0]
    reduced = [bool(getattr(t, "table_data_is_symmetry_reduced", False))
               for t in table_levels]
    if any(r != reduced[0] for r in reduced[1:]):
        raise RuntimeError("mixed full/reduced near-field table storage across levels")
    dtype = np.dtype(getattr(table0, "dtype", np.float64))
    info = _build_fast_scalar_arithmetic_orbit_reconstruction(table0)
    if info is None:
        return _prepare_dense_table_data(table_levels, reduced[0], dtype)
    layout = info["layout_entry_ids"]
    if len(layout) == 0:
        raise RuntimeError("near-field reconstruction layout contains no entries")
    for i, t in enumerate(table_levels):
        if not t.has_entry_data_for_full_indices(layout):
            raise RuntimeError(
                "near-field reconstruction layout references missing data" if i == 0 else
                "near-field levels disagree on reconstruction layout availability")
    tdc = np.zeros((len(table_levels), len(layout)), dtype=dtype)
    nm = np.zeros((len(table_levels), len(table0.mode_normalizers)),
                  dtype=table0.mode_normalizers.dtype)
    ext = np.zeros((len(table_levels), len(table0.kernel_exterior_normalizers)),
                   dtype=table0.kernel_exterior_normalizers.dtype)
    for lev, t in enumerate(table_levels):
        tdc[lev] = t.get_entry_data_for_full_indices(layout)
        nm[lev] = t.mode_normalizers
        ext[lev] = t.kernel_exterior_normalizers
    return (tdc, nm, ext, np.empty(0, dtype=np.int32), np.empty(0, dtype=dtype), info)


def _prepare_dense_table_data(table_levels, reduced, dtype):
    """The dense fallback (expansion_wrangler_fpnd.py:1887-1990, list1.py:
    1018-1048) for a kernel without an arithmetic orbit reconstruction: every
    level's full table, [level][case][source mode][target point], read as is
    by the device (``VL1_RECON_DENSE``).  A symmetry-reduced table of such a
    kernel would need the generated-orbit fallback, which is not built."""
    table0 = table_levels[0]
    if reduced:
        raise NotImplementedError(
            "this kernel has no arithmetic orbit reconstruction and its table is "
            "symmetry-reduced: the generated-orbit fallback (list1.py:903-1017) is not "
            "built; store the full table (the dense fallback)")
    n_full = int(table0.n_cases * table0.n_pairs)
    for t in table_levels:
        if t._data is None or np.asarray(t.data).size != n_full:
            raise RuntimeError("full near-field table has the wrong number of entries")
        if not np.all(np.isfinite(np.asarray(t.data))):
            raise RuntimeError("full near-field table contains non-finite entries")
    tdc = np.stack([np.asarray(t.data, dtype=dtype) for t in table_levels])
    nm = np.stack([np.asarray(t.mode_normalizers) for t in table_levels])
    ext = np.stack([np.asarray(t.kernel_exterior_normalizers) for t in table_levels])
    n_cases, dim = int(table0.n_cases), int(table0.dim)
    info = {
        "kind": "dense",
        # orbit arrays of the plan descriptor, not read for a dense table
        "case_orbit_ranks": np.zeros(n_cases, dtype=np.uint16),
        "case_axis_perm": np.zeros((n_cases, dim), dtype=np.uint8),
        "case_axis_sign": np.zeros((n_cases, dim), dtype=np.int8),
        "case_axis_group": np.zeros((n_cases, dim), dtype=np.uint8),
        "case_value_offsets": np.array([0, n_full], dtype=np.int32),
        "axis_sign_power": np.zeros(dim, dtype=np.uint8),
        "axis_direction_signs": np.zeros(dim, dtype=np.int8),
        "direction_sign_axis": -1,
        "layout_entry_ids": np.arange(n_full, dtype=np.int64),
        "layout_entry_scales": np.ones(n_full, dtype=np.int8),
        "n_case_orbits": 1,
        "metadata_bytes": 0,
        "compact_value_entry_count": n_full,
    }
    ids = np.arange(n_full, dtype=np.int32)
    return tdc, nm, ext, ids, np.ones(n_full, dtype=dtype), info


class FPNDTreeIndependentDataForWrangler:
    """Tree-independent wrangler data (target kernels, exclude_self)."""

    def __init__(self, cl_context=None, multipole_expansion_factory=None,
                 local_expansion_factory=None, target_kernels=(), exclude_self=True,
                 **kwargs):
        self.cl_context = cl_context
        self.multipole_expansion_factory = multipole_expansion_factory
        self.local_expansion_factory = local_expansion_factory
        self.target_kernels = tuple(target_kernels)
        self.exclude_self = exclude_self
        self.extra = kwargs


class _TimingFuture:
    def __init__(self, events):
        self.events = [e for e in events if e is not None]

    def result(self):
        return {}

    def done(self):
        return True

    def __call__(self):
        return 0.0


class FPNDExpansionWrangler(ExpansionWranglerInterface):
    """List-1 stage of the FPND wrangler on GB300.

    ``near_field_table``: a table, a per-level list of tables, or a dict
    ``{repr(kernel): table or list}`` (``expansion_wrangler_fpnd.py:2368-2404``).
    """

    def __init__(self, tree_indep, traversal, near_field_table, dtype=np.float64,
                 fmm_level_to_order=None, quad_order=None, potential_kind=1,
                 source_extra_kwargs=None, kernel_extra_kwargs=None,
                 self_extra_kwargs=None, list1_extra_kwargs=None, queue=None,
                 helmholtz_split=None, helmholtz_split_order=1,
                 helmholtz_split_smooth_quad_order=None,
                 helmholtz_split_order1_legacy_subtraction=False,
                 helmholtz_split_term_tables=None, helmholtz_split_auto_config=None,
                 **kwargs):
        self.tree_indep = tree_indep
        self.traversal = traversal
        self.tree = traversal.tree
        self.dtype = np.dtype(dtype)
        self.queue = queue
        self.potential_kind = potential_kind
        self.quad_order = quad_order
        self.source_extra_kwargs = source_extra_kwargs or {}
        self.kernel_extra_kwargs = kernel_extra_kwargs or {}
        self.self_extra_kwargs = self_extra_kwargs or {}
        self.list1_extra_kwargs = dict(list1_extra_kwargs or {})

        knames = [repr(k) for k in tree_indep.target_kernels]
        if isinstance(near_field_table, dict):
            tables = {}
            for kn in knames:
                if kn not in near_field_table:
                    raise RuntimeError(f"missing near-field table for kernel {kn}")
                v = near_field_table[kn]
                tables[kn] = list(v) if isinstance(v, (list, tuple)) else [v]
        else:
            v = near_field_table
            lst = list(v) if isinstance(v, (list, tuple)) else [v]
            tables = {kn: lst for kn in knames}
        self.near_field_table = tables
        for kn, lst in tables.items():
            self._check_table_levels(kn, lst)
        self._init_helmholtz_split(helmholtz_split, helmholtz_split_order,
                                   helmholtz_split_smooth_quad_order,
                                   helmholtz_split_order1_legacy_subtraction,
                                   helmholtz_split_term_tables, helmholtz_split_auto_config)
        self._payload_cache = collections.OrderedDict()
        self._payload_cache_max = 16
        self._view_cache = collections.OrderedDict()
        self._layout_validated = set()

    # {{{ Helmholtz split mode (expansion_wrangler_fpnd.py:2482-2600, 3491-3836)

    def _split_support(self):
        """(supported, reason): every target kernel Helmholtz, every table
        Laplace-backed."""
        for k in self.tree_indep.target_kernels:
            if type(base_kernel(k)).__name__ != "HelmholtzKernel":
                return False, f"target kernel {k!r} is not a Helmholtz kernel"
        for kn, lst in self.near_field_table.items():
            for t in lst:
                if type(t.integral_knl).__name__ != "LaplaceKernel":
                    return False, f"the near-field table of {kn} is not Laplace-backed"
        return True, ""

    def _init_helmholtz_split(self, split, order, smooth_quad_order, legacy, term_tables,
                              auto_config=None):
        from .helmholtz_split import choose_auto_split_order, split_rho_components

        ok, reason = self._split_support()
        if split is None:
            split = ok
        elif split and not ok:
            raise RuntimeError(
                "helmholtz_split requires Helmholtz target kernels and Laplace-backed "
                f"near-field tables; {reason}")
        self.helmholtz_split = bool(split)
        self._helmholtz_split_auto_config = dict(auto_config or {})
        self.helmholtz_split_auto_selection = None
        beta_mode = str(self._helmholtz_split_auto_config.get(
            "power_log_single_table_beta_mode", "p2p")).strip().lower()
        if beta_mode not in ("p2p", "table"):
            raise ValueError("power_log_single_table_beta_mode must be 'table' or 'p2p'")
        self._helmholtz_split_beta_mode = beta_mode
        auto = bool(self._helmholtz_split_auto_config.get("enabled", False)) or (
            isinstance(order, str) and order.strip().lower() == "auto")
        if self.helmholtz_split and auto:
            # expansion_wrangler_fpnd.py:2521-2575, 4252-4323: the order from
            # rho = |k| h_max of the coarsest box holding sources
            rho_r, rho_i = split_rho_components(
                self.tree, [self._split_wave_number(k) for k in self.tree_indep.target_kernels])
            order, info = choose_auto_split_order(self._helmholtz_split_auto_config, rho_r, rho_i)
            self.helmholtz_split_auto_selection = dict(info, order=order)
            if info["beyond_coverage"]:
                logger.warning("rho_max=%.3g exceeds the planner's threshold coverage; "
                               "split order clamped to %d", max(rho_r, rho_i), order)
        elif isinstance(order, str) and not auto:
            raise ValueError(f"helmholtz_split_order must be an integer or 'auto', got {order!r}")
        if self.helmholtz_split and int(order) > 1 and len(self.tree_indep.target_kernels) > 1:
            # the reference clamps to order 1 for several output kernels
            logger.warning("split order %d requested with %d target kernels; clamping to "
                           "order 1 for multi-output split mode", int(order),
                           len(self.tree_indep.target_kernels))
            order = 1
        self.helmholtz_split_order = int(order) if split else 1
        # extra term tables of split orders > 1, keyed ("power_log", 2n) in
        # 2D and ("power", 2j - 1) in 3D (expansion_wrangler_fpnd.py:2603-2647)
        self.helmholtz_split_term_tables = {}
        if term_tables is not None:
            if not isinstance(term_tables, dict):
                raise TypeError(
                    "helmholtz_split_term_tables must be a dict mapping term keys to tables")
            for key, tabs in term_tables.items():
                self.helmholtz_split_term_tables[_normalize_term_key(key)] = (
                    list(tabs) if isinstance(tabs, (list, tuple)) else [tabs])
        if self.helmholtz_split:
            if int(order) < 1:
                raise ValueError("helmholtz_split_order must be >= 1")
            if smooth_quad_order is not None:
                raise NotImplementedError("helmholtz_split_smooth_quad_order (resampled "
                                          "remainder sources) is not built")
            if legacy:
                raise NotImplementedError("the legacy order-1 subtraction is not built")

    def _split_wave_number(self, out_kernel):
        name = getattr(base_kernel(out_kernel), "helmholtz_k_name", "k")
        if name not in self.kernel_extra_kwargs:
            raise TypeError(f"missing kernel parameter {name!r} for "
                            f"{out_kernel.__class__.__name__} while evaluating split remainder")
        return complex(self.kernel_extra_kwargs[name])

    def _split_self_limit(self, k):
        """lim_{r->0} (G_k - G_0): 2D i/4 - (log(k/2) + gamma)/(2 pi), 3D i k/(4 pi)."""
        k = complex(k)
        if self.tree.dimensions == 3:
            return 1j * k / (4.0 * np.pi)
        if k == 0:
            return 0j
        return 0.25j - (np.log(0.5 * k) + np.euler_gamma) / (2.0 * np.pi)

    def _split_term_tables(self, out_kernel, key):
        """The term tables of ``key``: the given ones, else built on the GPU
        by the Duffy builder at the base tables' source box extents with the
        default term orders (expansion_wrangler_fpnd.py:4596-4619,
        4700-4775)."""
        from .helmholtz_split import term_build_orders, term_kernel
        from .nearfield_potential_table import NearFieldInteractionTable

        tabs = self.helmholtz_split_term_tables.get(key)
        if tabs is not None:
            return tabs
        base = self.near_field_table[repr(out_kernel)]
        dim = int(self.tree.dimensions)
        q = int(base[0].quad_order)
        reg, rad = term_build_orders(dim, q)
        knl = term_kernel(dim, key)
        tabs = []
        for t in base:
            tt = NearFieldInteractionTable(q, dim=dim, sumpy_kernel=knl,
                                           source_box_extent=float(t.source_box_extent))
            tt.build_table_via_duffy_radial(regular_quad_order=reg, radial_quad_order=rad,
                                            queue=self.queue)
            tabs.append(tt)
        self.helmholtz_split_term_tables[key] = tabs
        return tabs

    def _split_term_table_field(self, key, tabs, target_boxes, starts, lists, coefs):
        """The list-1 field of one term's table(s) for densities ``coefs``
        (expansion_wrangler_fpnd.py:4835-4907): a single table scaled by
        (h/h0)^(dim + power) without displacement, or one table per level;
        complex densities as real and imaginary parts."""
        import torch

        from .helmholtz_split import term_kernel, term_scaling_code
        from .plan import as_device_tensor

        dim = int(self.tree.dimensions)
        if len(tabs) > 1:
            l1kw = {"infer_kernel_scaling": False}
        else:
            l1kw = {"infer_kernel_scaling": False,
                    "kernel_scaling_code": term_scaling_code(dim, key[1]),
                    "kernel_displacement_code": "0.0"}
        knl = term_kernel(dim, key)
        payload = self.get_payload(knl, tabs)
        near_field = NearFieldFromCSR(knl, payload["table_data_shapes"],
                                      potential_kind=self.potential_kind, **l1kw)
        coefs = as_device_tensor(coefs)
        parts = [coefs.real, coefs.imag] if coefs.is_complex() else [coefs]
        vals = []
        for part in parts:
            kw = self._near_field_kwargs(payload, target_boxes, starts, lists,
                                         part.to(torch.float64).contiguous())
            res = torch.zeros(int(self.tree.ntargets), dtype=torch.float64, device="cuda")
            res, _ = near_field(self.queue, result=res, **kw)
            vals.append(res)
        field = vals[0].to(torch.complex128)
        if len(vals) > 1:
            field = field + 1j * vals[1]
        return field

    def _split_term_contribution(self, out_kernel, key, tabs, target_boxes, starts, lists,
                                 src_func, w, view, pts):
        """One term's list-1 contribution (expansion_wrangler_fpnd.py:
        3678-3806): the term table's near field, plus for a single
        r^{2n} log r table its log(h/h0) r^{2n} part - the point-to-point sum
        of r^{2n} with strengths x log(h/h0) (beta mode "p2p", the default),
        or the near field of the r^{2n} table for densities x log(h/h0)
        (beta mode "table", ``helmholtz_split_auto_config[
        "power_log_single_table_beta_mode"]``)."""
        import torch

        from .helmholtz_split import log_alpha_per_source, radial_power_sum
        from .plan import as_device_tensor, stream_handle

        kind, power = key
        dim = int(self.tree.dimensions)
        term = self._split_term_table_field(key, tabs, target_boxes, starts, lists, src_func)
        if dim == 2 and kind == "power_log" and len(tabs) == 1:
            beta = torch.from_numpy(log_alpha_per_source(
                self.tree, float(tabs[0].source_box_extent))).to("cuda")
            if self._helmholtz_split_beta_mode == "p2p":
                term = term + radial_power_sum(view, pts, w * beta, power,
                                               exclude_self=bool(self.tree_indep.exclude_self),
                                               stream=stream_handle(self.queue))
            else:
                pkey = ("power", power)
                ptabs = self._split_term_tables(out_kernel, pkey)
                dens = as_device_tensor(src_func)
                term = term + self._split_term_table_field(
                    pkey, ptabs, target_boxes, starts, lists, dens * beta.to(dens.dtype))
        return term

    def eval_direct_helmholtz_split_correction(self, target_boxes, neighbor_source_boxes_starts,
                                               neighbor_source_boxes_lists, src_weights,
                                               src_func=None):
        """The split mode's list-1 correction, one complex [N] array per
        target kernel (``expansion_wrangler_fpnd.py:3491-3836``): the
        remainder sum and, for split order p > 1, the extra terms' table
        contributions times their coefficients (``src_func``: the density at
        the points, needed for p > 1).  ``src_weights``: density x quadrature
        weight in tree order."""
        import torch

        from .helmholtz_split import (
            max_neighbor_distance,
            series_terms,
            split_correction,
            split_extra_terms,
        )
        from .plan import as_device_tensor, stream_handle, tree_view_from_arrays

        if not self.helmholtz_split:
            return self.output_zeros(), _TimingFuture([])
        order = int(self.helmholtz_split_order)
        if order > 1 and src_func is None:
            raise ValueError("split orders above 1 need the density (src_func) for the "
                             "extra term tables")
        w = as_device_tensor(src_weights)
        pts = torch.from_numpy(np.ascontiguousarray(_np(self.tree.sources),
                                                    dtype=np.float64)).to("cuda")
        out, events = [], []
        r_max = max_neighbor_distance(self.tree)
        for k in self.tree_indep.target_kernels:
            kw = self._near_field_kwargs(self.get_payload(k), target_boxes,
                                         neighbor_source_boxes_starts,
                                         neighbor_source_boxes_lists, None)
            view, keep = tree_view_from_arrays(**{n: kw[n] for n in (
                "target_boxes", "neighbor_source_boxes_starts", "neighbor_source_boxes_lists",
                "box_centers", "box_levels", "box_source_starts",
                "box_source_counts_nonchild", "box_target_starts",
                "box_target_counts_nonchild", "source_mode_ids", "target_point_ids",
                "root_extent")})
            wave = self._split_wave_number(k)
            exclude = bool(self.tree_indep.exclude_self)
            corr = split_correction(view, pts, w, wave, series_terms(self.tree.dimensions,
                                                                     wave, r_max),
                                    exclude_self=exclude, stream=stream_handle(self.queue),
                                    split_order=order)
            for key, coeff in split_extra_terms(self.tree.dimensions, wave, order):
                tabs = self._split_term_tables(k, key)
                corr = corr + coeff * self._split_term_contribution(
                    k, key, tabs, target_boxes, neighbor_source_boxes_starts,
                    neighbor_source_boxes_lists, src_func, w, view, pts)
            if exclude:
                # self pairs excluded from the sum: add back the finite r -> 0
                # limit of the remainder per point (expansion_wrangler_fpnd.py:
                # 3824-3833, 5293-5360)
                corr = corr + w.to(torch.complex128) * self._split_self_limit(wave)
            evt = torch.cuda.Event()
            evt.record()
            out.append(corr)
            events.append(evt)
            del keep
        return out, _TimingFuture(events)

    # }}}

    # {{{ table bookkeeping (expansion_wrangler_fpnd.py:2414-2472)

    def _check_table_levels(self, kname, tables):
        t0 = tables[0]
        root = float(self.tree.root_extent)
        for lev, t in enumerate(tables):
            expected = float(t0.source_box_extent) * 0.5 ** lev
            if not math.isclose(float(t.source_box_extent), expected, rel_tol=1e-12):
                raise RuntimeError(
                    f"near-field tables for {kname} must halve the source box extent per "
                    f"level: level {lev} has {t.source_box_extent}, expected {expected}")
        ratio = root / float(t0.source_box_extent)
        if ratio <= 0:
            raise RuntimeError("invalid table source_box_extent")

    def table_starting_level(self, table0):
        return int(np.round(np.log(float(self.tree.root_extent)
                                   / float(table0.source_box_extent)) / np.log(2)))

    # }}}

    def eval_dtype(self, out_kernel):
        cfg = self.dtype
        if out_kernel.is_complex_valued:
            return cfg if cfg.kind == "c" else (
                np.dtype(np.complex64) if cfg == np.float32 else np.dtype(np.complex128))
        return cfg if cfg.kind == "f" else (
            np.dtype(np.float32) if cfg == np.complex64 else np.dtype(np.float64))

    def get_payload(self, out_kernel, tables=None):
        """Device-ready payload of ``out_kernel``'s tables (LRU of 16)."""
        kname = repr(out_kernel)
        tables = tables or self.near_field_table[kname]
        eval_dtype = self.eval_dtype(out_kernel)
        if getattr(self, "helmholtz_split", False):
            # split mode: the Laplace tables' real values (the remainder sum
            # adds the complex part)
            eval_dtype = np.dtype(np.float64)
        key = (kname, tuple(id(t) for t in tables),
               tuple(int(np.asarray(t.data).ctypes.data) for t in tables),
               tuple(int(np.asarray(t.data).size) for t in tables), eval_dtype.str)
        hit = self._payload_cache.get(key)
        if hit is not None:
            self._payload_cache.move_to_end(key)
            return hit
        table0 = tables[0]
        vals = sorted({int(c) for v in table0.interaction_case_vecs for c in v})
        base, shift = vals[-1] - vals[0] + 1, -vals[0]
        tdc, nm, ext, _, _, info = _prepare_table_data_and_entry_map(tables)
        if eval_dtype.kind != "c" and np.iscomplexobj(tdc):
            raise TypeError("complex table data for a real-valued output kernel")
        tdc = tdc.astype(eval_dtype)
        nm = nm.astype(eval_dtype)
        ext = ext.astype(eval_dtype)
        shapes = {
            "n_tables": len(tables), "quad_order": table0.quad_order,
            "n_q_points": table0.n_q_points, "n_cases": table0.n_cases,
            "n_table_entries": tdc.shape[1], "reconstruction_kind": info["kind"],
            "n_arithmetic_case_orbits": int(info["n_case_orbits"]),
        }
        payload = {
            "base": base, "shift": shift, "case_indices": np.asarray(table0.case_indices),
            "table_data": tdc, "mode_nmlz": nm, "exterior_mode_nmlz": ext,
            "table_data_shapes": shapes, "reconstruction_info": info,
            "table_root_extent": float(table0.source_box_extent),
            "table_starting_level": self.table_starting_level(table0),
            "reconstruction_diagnostics": {
                "kind": info["kind"],
                "online_value_bytes": int(tdc.nbytes),
                "generated_reconstruction_metadata_bytes": int(info["metadata_bytes"]),
                "normalizer_auxiliary_bytes": int(nm.nbytes + ext.nbytes),
                "value_dense_block_equivalents": float(tdc.shape[1] / table0.n_pairs),
            },
        }
        self._payload_cache[key] = payload
        while len(self._payload_cache) > self._payload_cache_max:
            self._payload_cache.popitem(last=False)
        return payload

    def _near_field_kwargs(self, payload, target_boxes, starts, lists, mode_coefs):
        tree = self.tree
        nq = payload["table_data_shapes"]["n_q_points"]
        local = _compute_box_local_ids(tree, nq)
        key = (id(target_boxes), id(lists), nq)
        if key not in self._layout_validated:
            _validate_table_box_particle_layout(tree, target_boxes, lists, nq)
            self._layout_validated.add(key)
        info = payload["reconstruction_info"]
        counts = _np(tree.box_target_counts_nonchild).astype(np.int32)
        return dict(
            box_centers=tree.box_centers, box_levels=tree.box_levels,
            box_source_counts_nonchild=counts, box_source_starts=tree.box_target_starts,
            box_target_counts_nonchild=counts, box_target_starts=tree.box_target_starts,
            case_indices=payload["case_indices"], encoding_base=payload["base"],
            encoding_shift=payload["shift"], mode_nmlz_combined=payload["mode_nmlz"],
            exterior_mode_nmlz_combined=payload["exterior_mode_nmlz"],
            neighbor_source_boxes_starts=starts, root_extent=tree.root_extent,
            neighbor_source_boxes_lists=lists, mode_coefs=mode_coefs,
            source_mode_ids=local, table_data_combined=payload["table_data"],
            target_boxes=target_boxes, target_point_ids=local,
            table_root_extent=payload["table_root_extent"],
            table_starting_level=payload["table_starting_level"],
            arithmetic_case_orbit_ranks=info["case_orbit_ranks"],
            arithmetic_case_axis_perm=info["case_axis_perm"],
            arithmetic_case_axis_sign=info["case_axis_sign"],
            arithmetic_case_axis_group=info["case_axis_group"],
            arithmetic_case_value_offsets=info["case_value_offsets"],
            arithmetic_axis_sign_power=info["axis_sign_power"],
            arithmetic_axis_direction_signs=info["axis_direction_signs"],
            arithmetic_direction_sign_axis=info["direction_sign_axis"])

    def near_field_evaluator(self, out_kernel, payload, list1_extra_kwargs=None):
        kw = dict(self.list1_extra_kwargs if list1_extra_kwargs is None
                  else list1_extra_kwargs)
        if self.helmholtz_split:
            # the Laplace-table part with the split scaling rules
            # (expansion_wrangler_fpnd.py:4801-4833)
            from .helmholtz_split import split_scaling_codes
            from .kernels import LaplaceKernel

            scaling, disp = split_scaling_codes(self.tree.dimensions)
            kw.setdefault("kernel_scaling_code", scaling)
            kw.setdefault("kernel_displacement_code", disp)
            return NearFieldFromCSR(LaplaceKernel(self.tree.dimensions),
                                    payload["table_data_shapes"],
                                    potential_kind=self.potential_kind, **kw)
        return NearFieldFromCSR(out_kernel, payload["table_data_shapes"],
                                potential_kind=self.potential_kind, **kw)

    def eval_direct_single_out_kernel(self, out_pot, out_kernel, target_boxes,
                                      neighbor_source_boxes_starts,
                                      neighbor_source_boxes_lists, mode_coefs,
                                      near_field_tables=None, list1_extra_kwargs=None):
        payload = self.get_payload(out_kernel, near_field_tables)
        tables = near_field_tables or self.near_field_table[repr(out_kernel)]
        if len(tables) > 1:
            min_lev = int(np.min(_np(self.tree.box_levels)[_np(target_boxes).astype(np.int64)]))
            largest = float(self.tree.root_extent) * 0.5 ** min_lev
            if not float(tables[0].source_box_extent) >= largest - 1e-15:
                raise RuntimeError(
                    "Insufficient list of tables: the coarsest level mesh cells at level "
                    f"{min_lev} are not covered.")
        near_field = self.near_field_evaluator(out_kernel, payload, list1_extra_kwargs)
        kw = self._near_field_kwargs(payload, target_boxes, neighbor_source_boxes_starts,
                                     neighbor_source_boxes_lists, mode_coefs)
        if self.helmholtz_split and out_pot.is_complex():
            import torch

            real = torch.zeros(out_pot.shape, dtype=torch.float64, device=out_pot.device)
            res, evt = near_field(self.queue, result=real, **kw)
            out_pot.copy_(res)
            return out_pot, evt
        res, evt = near_field(self.queue, result=out_pot, **kw)
        return res, evt

    def output_zeros(self):
        import torch
        n = int(self.tree.ntargets)
        out = []
        for k in self.tree_indep.target_kernels:
            dt = torch.complex128 if self.eval_dtype(k).kind == "c" else torch.float64
            out.append(torch.zeros(n, dtype=dt, device="cuda"))
        return out

    def eval_direct(self, target_boxes, neighbor_source_boxes_starts,
                    neighbor_source_boxes_lists, mode_coefs):
        from .plan import as_device_tensor
        pot = self.output_zeros()
        coefs = as_device_tensor(mode_coefs)
        events = []
        for i, k in enumerate(self.tree_indep.target_kernels):
            pot[i], evt = self.eval_direct_single_out_kernel(
                pot[i], k, target_boxes, neighbor_source_boxes_starts,
                neighbor_source_boxes_lists, coefs)
            events.append(evt)
        return pot, _TimingFuture(events)

    def eval_direct_batched(self, target_boxes, neighbor_source_boxes_starts,
                            neighbor_source_boxes_lists, mode_coefs, *, precision="fp64"):
        """All right-hand sides at once: ``mode_coefs`` is ``[nrhs, N]``.

        Returns one ``[nrhs, N]`` tensor per target kernel (per-RHS outputs).
        ``precision`` is ``"fp64"`` (FP64 kernel) or ``"mixed"`` (tensor-core
        contraction with exact split products, see ``batched.py``).
        """
        import torch

        from .plan import as_device_tensor, stream_handle, tree_view_from_arrays
        coefs = as_device_tensor(mode_coefs)
        if coefs.dim() == 1:
            coefs = coefs[None, :]
        nrhs = int(coefs.shape[0])
        outs, events = [], []
        for k in self.tree_indep.target_kernels:
            payload = self.get_payload(k)
            nf = self.near_field_evaluator(k, payload)
            kw = self._near_field_kwargs(payload, target_boxes, neighbor_source_boxes_starts,
                                         neighbor_source_boxes_lists, None)
            plan = nf.get_plan(
                table_data_combined=kw["table_data_combined"],
                mode_nmlz_combined=kw["mode_nmlz_combined"], case_indices=kw["case_indices"],
                encoding_base=kw["encoding_base"], encoding_shift=kw["encoding_shift"],
                table_root_extent=kw["table_root_extent"],
                table_starting_level=kw["table_starting_level"],
                **{n: kw[n] for n in kw if n.startswith("arithmetic_")})
            nf._check_single_table_levels(kw["neighbor_source_boxes_lists"],
                                          kw["box_levels"], kw["table_starting_level"])
            # device tree arrays per (box lists, layout): repeated calls reuse
            # them, and with them the cached tensor-core schedule
            vkey = (id(target_boxes), id(neighbor_source_boxes_starts),
                    id(neighbor_source_boxes_lists), int(payload["table_data_shapes"]
                                                         ["n_q_points"]))
            hit = self._view_cache.get(vkey)
            if hit is None or hit[2] is not target_boxes:
                view, keep = tree_view_from_arrays(**{n: kw[n] for n in (
                    "target_boxes", "neighbor_source_boxes_starts",
                    "neighbor_source_boxes_lists", "box_centers", "box_levels",
                    "box_source_starts", "box_source_counts_nonchild", "box_target_starts",
                    "box_target_counts_nonchild", "source_mode_ids", "target_point_ids",
                    "root_extent")})
                if len(self._view_cache) >= 4:
                    self._view_cache.pop(next(iter(self._view_cache)))
                self._view_cache[vkey] = (view, keep, target_boxes)
            else:
                view, keep = hit[0], hit[1]
            c = coefs
            if c.dtype not in (torch.float64, torch.complex128):
                c = c.to(torch.complex128 if c.is_complex() else torch.float64)
            c = c.contiguous()
            out_complex = plan.complex_table or c.is_complex()
            out = torch.empty((nrhs, int(view.n_particles)),
                              dtype=torch.complex128 if out_complex else torch.float64,
                              device="cuda")
            stream = stream_handle(self.queue)
            if precision == "fp64":
                plan.eval_fp64(view, c, out, stream=stream, nrhs=nrhs)
            else:
                from .batched import eval_mixed
                eval_mixed(plan, view, c, out, stream=stream, nrhs=nrhs, keep=keep)
            evt = torch.cuda.Event()
            evt.record()
            plan.raise_on_status(stream)
            outs.append(out)
            events.append(evt)
        return outs, _TimingFuture(events)

    # {{{ reordering and bookkeeping of drive_volume_fmm

    def reorder_sources(self, source_array):
        from .plan import as_device_tensor
        x = as_device_tensor(source_array)
        idx = as_device_tensor(_np(self.tree.user_source_ids).astype(np.int64))
        return x[..., idx]

    def reorder_targets(self, target_array):
        return self.reorder_sources(target_array)

    def reorder_potentials(self, potentials):
        from .plan import as_device_tensor
        idx = as_device_tensor(_np(self.tree.sorted_target_ids).astype(np.int64))
        return [p[..., idx] for p in potentials]

    def finalize_potentials(self, potentials):
        return potentials

    def form_multipoles(self, level_start_source_box_nrs, source_boxes, src_weights):
        # far field is outside the list-1 path; drive_volume_fmm(list1_only=True)
        # discards it in the reference as well
        return None, None

    def coarsen_multipoles(self, level_start_source_parent_box_nrs, source_parent_boxes,
                           mpoles):
        return mpoles, None

    # }}}


FPNDSumpyExpansionWrangler = FPNDExpansionWrangler
