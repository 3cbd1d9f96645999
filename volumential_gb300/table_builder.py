"""FP64 GPU builder of near-field table values (Duffy radial quadrature).

The reference fills a table with ``build_table_via_duffy_radial``
(``volumential/nearfield_potential_table.py:2948-3195``), whose default path
evaluates every orbit-invariant entry with one generated OpenCL kernel
(``:2035-2223``, ``:2331-2463``) over the node set of ``:2225-2291``.  This
module assembles the same per-entry geometry (target point of the case,
target clipped to the source box, the source mode's per-axis indices) and the
1D rules, and calls ``vl1_duffy_table`` (``include/vl1.h``), which decodes the
Duffy node set on the device and sums in FP64.

1D rules (restated from ``volumential/singular_integral_2d.py:807-853``):
``tanh-sinh-fast`` with n = max(3, order) is the tanh-sinh rule on [0, 1]
with step h = 1/sqrt(n) over the integers -n..n, x = (1 + tanh(pi/2 sinh t))/2,
w = pi/4 h cosh t sech^2(pi/2 sinh t), keeping nodes strictly inside (0, 1);
``tanh-sinh`` takes mpmath's tanh-sinh nodes of degree max(3, order // 5)
mapped to [0, 1]; the tail rule is Gauss-Legendre on [0, 1], tensor in
dimension 3 (first tail axis slowest).

Kernels (``G`` includes the scaling constant; the reference takes both from
sumpy, which is not available here, so these are the standard free-space
Green's functions): Laplace 2D -log(r)/(2 pi), 3D 1/(4 pi r); Helmholtz 2D
(i/4) H0^(1)(k r), 3D exp(i k r)/(4 pi r); constant 1.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib

__all__ = ["tanh_sinh_fast_rule", "radial_rule", "gauss_legendre_unit", "regular_rule",
           "lagrange_product_weights", "entry_geometry", "kernel_code",
           "build_table_values", "DEFAULT_ORDERS", "DuffyBuildConfig", "DEFAULT_ORDER_CANDIDATES",
           "is_auto_order", "select_duffy_orders", "autotune_duffy_orders"]

#: the reference's defaults (``nearfield_potential_table.py:2948-2953``)
DEFAULT_ORDERS = {"regular_quad_order": 20, "radial_quad_order": 61}


def tanh_sinh_fast_rule(order):
    """Tanh-sinh nodes and weights on (0, 1) with n = max(3, order) steps of
    h = 1/sqrt(n) on each side (the reference's ``tanh-sinh-fast``)."""
    n = max(3, int(order))
    h = 1.0 / np.sqrt(n)
    t = h * np.arange(-n, n + 1, dtype=np.float64)
    a = 0.5 * np.pi * np.sinh(t)
    x = 0.5 * (1.0 + np.tanh(a))
    # sech^2(a) = 4 e^{-2|a|} / (1 + e^{-2|a|})^2, without overflow
    e = np.exp(-2.0 * np.abs(a))
    w = 0.25 * np.pi * h * np.cosh(t) * (4.0 * e / (1.0 + e) ** 2)
    keep = (x > 0.0) & (x < 1.0) & np.isfinite(w)
    return x[keep], w[keep]


def radial_rule(rule, order, mp_dps=50):
    if rule == "tanh-sinh-fast":
        return tanh_sinh_fast_rule(order)
    if rule == "tanh-sinh":
        import mpmath

        old = mpmath.mp.dps
        mpmath.mp.dps = mp_dps
        try:
            ts = mpmath.calculus.quadrature.TanhSinh(mpmath.mp)
            prec = int(np.log(10) / np.log(2) * mpmath.mp.dps)
            nodes = ts.calc_nodes(degree=max(3, int(order // 5)), prec=prec)
            x = np.array([float(p[0]) for p in nodes])
            w = np.array([float(p[1]) for p in nodes])
        finally:
            mpmath.mp.dps = old
        return 0.5 * (x + 1.0), 0.5 * w
    raise ValueError(f"unsupported radial rule {rule!r} (tanh-sinh-fast or tanh-sinh)")


def gauss_legendre_unit(order):
    """Gauss-Legendre rule on [0, 1] (scipy's nodes, as the reference's)."""
    from scipy.special import roots_legendre

    x, w = roots_legendre(int(order))
    return 0.5 * (x + 1.0), 0.5 * w


def regular_rule(dim_minus_one, order):
    """Tensor Gauss-Legendre tail rule on [0, 1]^(dim - 1): (nodes [n, dim - 1],
    weights [n]), first tail axis slowest."""
    if dim_minus_one == 0:
        return np.zeros((1, 0)), np.ones(1)
    x, w = gauss_legendre_unit(order)
    grids = np.meshgrid(*([x] * dim_minus_one), indexing="ij")
    wgrids = np.meshgrid(*([w] * dim_minus_one), indexing="ij")
    return (np.stack([g.ravel() for g in grids], axis=-1),
            np.prod(np.array(wgrids), axis=0).ravel())


def lagrange_product_weights(xi):
    """1 / prod_{j != m} (x_m - x_j): the Lagrange polynomial of node m is
    w_m prod_{j != m} (x - x_j)."""
    xi = np.asarray(xi, dtype=np.float64)
    d = xi[:, None] - xi[None, :]
    np.fill_diagonal(d, 1.0)
    return 1.0 / np.prod(d, axis=1)


def entry_geometry(table, entry_ids):
    """Per entry: target point [dim, n], target clipped to the source box
    [dim, n] and source mode index per axis [dim, n] (axis 0 slowest)."""
    entry_ids = np.asarray(entry_ids, dtype=np.int64)
    case = entry_ids // table.n_pairs
    pair = entry_ids % table.n_pairs
    smode = pair // table.n_q_points
    tpoint = pair % table.n_q_points
    tp = table.get_case_target_points()[:, case, tpoint]
    dc = np.clip(tp, 0.0, table.source_box_extent)
    q, dim = table.quad_order, table.dim
    axes = np.empty((dim, len(entry_ids)), dtype=np.int32)
    rem = smode.copy()
    for a in range(dim - 1, -1, -1):
        axes[a] = rem % q
        rem //= q
    return np.ascontiguousarray(tp), np.ascontiguousarray(dc), axes


def kernel_derivative(knl):
    """(base kernel, derivative code) of a kernel: 0 for an undifferentiated
    one, a + 1 for ``AxisTargetDerivative(a, .)``, -(a + 1) for
    ``AxisSourceDerivative(a, .)`` (first derivatives only)."""
    name = type(knl).__name__
    if name in ("AxisTargetDerivative", "AxisSourceDerivative"):
        inner = knl.inner_kernel
        if hasattr(inner, "inner_kernel"):
            raise NotImplementedError("the GPU Duffy builder takes first derivatives only")
        a = int(knl.axis)
        return inner, (a + 1) if name == "AxisTargetDerivative" else -(a + 1)
    return knl, 0


def kernel_code(table, kernel=None):
    """(vl1 kernel code, complex) of a table's kernel or of an explicit
    ``kernel`` name ("laplace", "helmholtz", "constant", "plane_wave",
    "power", "power_log")."""
    if kernel is None:
        if table.kernel_type == "const":
            kernel = "constant"
        else:
            base = (kernel_derivative(table.integral_knl)[0]
                    if table.integral_knl is not None else None)
            name = type(base).__name__ if base is not None else ""
            kernel = {"LaplaceKernel": "laplace", "HelmholtzKernel": "helmholtz",
                      "ConstantKernel": "constant", "PlaneWaveKernel": "plane_wave",
                      "RadialPowerKernel": "power",
                      "_RadialPowerKernel": "power", "RadialPowerLogKernel": "power_log",
                      "_RadialPowerLogKernel": "power_log"}.get(name)
            if kernel is None:
                raise NotImplementedError(
                    f"no GPU Duffy kernel for {name or table.kernel_type!r} (Laplace, "
                    "Helmholtz, constant and radial power kernels are built)")
    if kernel == "power":
        return _lib.VL1_DUFFY_POWER, False
    if kernel == "power_log":
        return _lib.VL1_DUFFY_POWER_LOG, False
    dim = table.dim
    if kernel == "laplace":
        return (_lib.VL1_DUFFY_LAPLACE2D if dim == 2 else _lib.VL1_DUFFY_LAPLACE3D), False
    if kernel == "helmholtz":
        return (_lib.VL1_DUFFY_HELMHOLTZ2D if dim == 2 else _lib.VL1_DUFFY_HELMHOLTZ3D), True
    if kernel == "constant":
        return _lib.VL1_DUFFY_CONSTANT, False
    if kernel == "plane_wave":
        return _lib.VL1_DUFFY_PLANE_WAVE, False
    raise ValueError(f"unknown kernel {kernel!r}")


def build_table_values(table, *, radial_rule_name="tanh-sinh-fast", regular_quad_order=20,
                       radial_quad_order=61, mp_dps=50, kernel=None, k=None,
                       entry_ids=None, stream=None, store=True, max_ctas=0, power=None):
    """Compute the table's orbit-invariant entries on the GPU (FP64) and, with
    ``store``, keep them as its compact data (plus the 2D normalizers).
    ``max_ctas`` > 0 runs the build on at most that many CTAs (a build in the
    background of other GPU work); ``power``: the radial power kernels'
    power (default: the table kernel's).  Returns (entry_ids, values)."""
    import torch

    from .plan import require_cuda

    require_cuda()
    code, cplx = kernel_code(table, kernel)
    if code in (_lib.VL1_DUFFY_HELMHOLTZ2D, _lib.VL1_DUFFY_HELMHOLTZ3D,
                _lib.VL1_DUFFY_PLANE_WAVE):
        if k is None:
            base = kernel_derivative(table.integral_knl)[0]
            name = getattr(base, "helmholtz_k_name", getattr(base, "plane_wave_k_name", "k"))
            k = table.build_extra_kwargs.get(name)
        if k is None or not np.isfinite(k):
            raise ValueError("a finite wave number k is required for this kernel")
    if code in (_lib.VL1_DUFFY_POWER, _lib.VL1_DUFFY_POWER_LOG):
        if power is None:
            power = getattr(table.integral_knl, "power", None)
        if power is None:
            raise ValueError("the radial power kernels need a power")
    if cplx and not np.issubdtype(np.dtype(table.dtype), np.complexfloating):
        raise TypeError("complex kernel values need a complex table dtype")
    full = False
    if entry_ids is None:
        if table.dim not in (2, 3):
            raise NotImplementedError("tables of dimension 2 and 3 only")
        info = table._get_invariant_entry_info()
        if info is None:   # no orbit symmetry: every entry (a dense table)
            entry_ids = np.arange(table.n_cases * table.n_pairs, dtype=np.int64)
            full = True
        else:
            entry_ids = info["entry_ids"]
    entry_ids = np.asarray(entry_ids, dtype=np.int64)
    if entry_ids.size and (entry_ids.min() < 0 or entry_ids.max() >= table.n_cases *
                           table.n_pairs):
        raise ValueError("entry ids outside the table")
    tp, dc, axes = entry_geometry(table, entry_ids)
    rx, rw = radial_rule(radial_rule_name, radial_quad_order, mp_dps)
    gx, gw = gauss_legendre_unit(regular_quad_order)
    xi = np.asarray(table.q_points[:table.quad_order, table.dim - 1], dtype=np.float64)
    bw = lagrange_product_weights(xi)

    dev = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(  # noqa: E731
        device="cuda", dtype=dt)
    arrs = {"tp": dev(tp), "dc": dev(dc), "ax": dev(axes, torch.int32), "gx": dev(gx),
            "gw": dev(gw), "rx": dev(rx), "rw": dev(rw), "xi": dev(xi), "bw": dev(bw)}
    n = len(entry_ids)
    out = torch.empty((n, 2) if cplx else (n,), dtype=torch.float64, device="cuda")
    d = _lib.DuffyDesc()
    d.dim, d.q, d.n_entries = table.dim, table.quad_order, n
    d.n_reg, d.n_rad, d.kernel = len(gx), len(rx), code
    d.complex_output = int(cplx)
    d.max_ctas = int(max_ctas)
    d.power = int(power or 0)
    d.derivative = (kernel_derivative(table.integral_knl)[1]
                    if table.integral_knl is not None else 0)
    d.extent = float(table.source_box_extent)
    d.k = float(k) if k is not None else 0.0
    d.target_points, d.decomposition_targets = arrs["tp"].data_ptr(), arrs["dc"].data_ptr()
    d.mode_axes = arrs["ax"].data_ptr()
    d.regular_nodes, d.regular_weights = arrs["gx"].data_ptr(), arrs["gw"].data_ptr()
    d.radial_nodes, d.radial_weights = arrs["rx"].data_ptr(), arrs["rw"].data_ptr()
    d.interp_nodes, d.interp_weights = arrs["xi"].data_ptr(), arrs["bw"].data_ptr()
    sh = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.lib().vl1_duffy_table(C.byref(d), C.c_void_p(out.data_ptr() if n else 0),
                                          C.c_void_p(sh)), "vl1_duffy_table")
    # wait for the build on its stream first: a device-to-host copy queued
    # behind the build kernel holds up other host threads' CUDA calls (a
    # serving loop's launches) until the kernel finishes
    torch.cuda.ExternalStream(sh).synchronize()
    vals = out.cpu().numpy()
    if cplx:
        vals = vals[:, 0] + 1j * vals[:, 1]
    if not np.all(np.isfinite(vals)):
        raise RuntimeError("the Duffy builder produced non-finite table values")
    if store and full:
        table.data = vals.astype(table.dtype)
        table.is_built = True
        if table.dim == 2:
            table.build_normalizer_table()
    elif store:
        table.set_reduced_table_data(entry_ids, vals.astype(table.dtype))
        if table.dim == 2:
            table.build_normalizer_table()
    return entry_ids, vals


# {{{ Duffy order selection (nearfield_potential_table.py:195-206, 2301-2326, 2465-2619)

@dataclass(frozen=True)
class DuffyBuildConfig:
    """Build settings of a Duffy table (the reference's dataclass of the same
    name): orders may be ``"auto"`` / ``None``, or ``auto_tune_orders`` set,
    to choose them by convergence on sample entries."""
    radial_rule: str = "tanh-sinh-fast"
    regular_quad_order: object = 20
    radial_quad_order: object = 61
    mp_dps: int = 50
    auto_tune_orders: bool = False
    auto_tune_samples: int = 5
    auto_tune_floor_factor: float = 8.0
    auto_tune_candidates: object = None


#: (regular, radial) candidates of dimensions 2 and 3, in increasing cost
DEFAULT_ORDER_CANDIDATES = ((4, 11), (4, 21), (6, 21), (6, 31), (8, 31), (10, 41), (12, 61))


def is_auto_order(value):
    return value is None or (isinstance(value, str) and value.strip().lower() == "auto")


def select_duffy_orders(candidates, candidate_values, floor_factor=8.0):
    """Index of the cheapest candidate within the convergence floor, and the
    diagnostics.  Errors are taken against the last (most accurate)
    candidate, relative to max(1, |reference|) per entry; the floor is the
    smallest positive error among the (up to three) candidates before the
    last, at least 128 eps; a candidate is accepted within ``floor_factor``
    times the floor (nearfield_potential_table.py:2576-2598)."""
    ref = np.asarray(candidate_values[-1])
    denom = np.maximum(1.0, np.abs(ref))
    errs = [float(np.max(np.abs(np.asarray(v) - ref) / denom)) if ref.size else 0.0
            for v in candidate_values]
    floor = 0.0
    if len(errs) > 2:
        tail = np.asarray(errs[max(0, len(errs) - 4):-1], dtype=np.float64)
        pos = tail[tail > 0]
        if pos.size >= 2:
            floor = float(np.min(pos))
    floor = max(floor, 128.0 * np.finfo(np.float64).eps)
    threshold = float(floor_factor) * floor
    sel = len(candidates) - 1
    for i, e in enumerate(errs):
        if e <= threshold:
            sel = i
            break
    return sel, {"relative_errors_vs_best": errs, "floor_estimate": floor,
                 "acceptance_threshold": threshold}


def autotune_duffy_orders(table, *, radial_rule="tanh-sinh-fast", mp_dps=50, sample_count=5,
                          candidates=None, floor_factor=8.0, kernel=None, k=None,
                          stream=None):
    """Choose (regular, radial) orders for ``table``: its sample entries
    (evenly spaced over the entries to build) evaluated on the GPU at every
    candidate, the first within the convergence floor kept.  Returns
    (regular, radial, info)."""
    if radial_rule == "adaptive":
        raise ValueError("Duffy order auto-tuning is only available for fixed radial rules")
    cands = [tuple(int(x) for x in pair)
             for pair in (DEFAULT_ORDER_CANDIDATES if candidates is None else candidates)]
    if not cands:
        raise ValueError("Duffy order auto-tuning candidate list cannot be empty")
    info = table._get_invariant_entry_info()
    ids = (np.asarray(info["entry_ids"], dtype=np.int64) if info is not None
           else np.arange(table.n_cases * table.n_pairs, dtype=np.int64))
    if ids.size == 0:
        sample = ids
    elif int(sample_count) >= ids.size:
        sample = ids
    else:
        sample = ids[np.unique(np.linspace(0, ids.size - 1, num=max(1, int(sample_count)),
                                           dtype=np.int64))]
    values = []
    for reg, rad in cands:
        if sample.size:
            _, v = build_table_values(table, radial_rule_name=radial_rule,
                                      regular_quad_order=reg, radial_quad_order=rad,
                                      mp_dps=mp_dps, kernel=kernel, k=k, entry_ids=sample,
                                      stream=stream, store=False)
        else:
            v = np.zeros(0)
        values.append(v)
    sel, diag = select_duffy_orders(cands, values, floor_factor)
    out = {"auto_tuned": True, "selected_regular_quad_order": cands[sel][0],
           "selected_radial_quad_order": cands[sel][1],
           "sample_entry_ids": [int(e) for e in sample], "candidates": cands}
    out.update(diag)
    return cands[sel][0], cands[sel][1], out

# }}}
