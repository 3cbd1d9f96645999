"""Helmholtz split mode: Laplace-table near field plus a list-1 remainder sum.

The reference's default Helmholtz list-1 evaluation
(``volumential/expansion_wrangler_fpnd.py:2482-2519, 3491-3836``) uses the
Laplace table (scaled by the split rules of ``:4801-4833``) and adds, per
target, the sum over list-1 source points of (density x quadrature weight)
x R(r), with R = G_k - G_0 the smooth Helmholtz-minus-Laplace remainder.  For
split order 1 (the default) R is the series of ``:212-332``:

* 2D: R = c0 + sum_{n>=1} (a_n log r + b_n) r^{2n} with
  c0 = i/4 - (log(k/2) + gamma) / (2 pi), s_n = (-1)^n (k^2/4)^n / (n!)^2,
  a_n = -s_n / (2 pi), b_n = s_n ((H_n - log(k/2) - gamma) / (2 pi) + i/4);
* 3D: R = sum_{n>=1} (i k)^n / (4 pi n!) r^{n-1}  ( = (e^{ikr} - 1) / (4 pi r) ),

truncated at the term count of ``:4337-4378`` (tolerance 1e-16 at the largest
list-1 distance, at most 96 terms, plus 2).  ``split_correction`` evaluates
the sum on the GPU (``vl1_split_correction``).

Split order p > 1 (``:212-332, 4552-4570, 5052-5115``) moves the non-smooth
terms of the first p - 1 orders out of R into near-field tables of their
own kernels, integrated by the Duffy builder instead of point quadrature:
2D r^{2n} log r (n = 1..p-1, coefficient a_n), 3D r^{2j-1} (j = 1..p-1,
coefficient c_{2j}).  A single term table of source box extent h0 serves
every level through the scaling (h/h0)^(dim + power)
(``:4777-4799``); for r^{2n} log r the remaining log(h/h0) r^{2n} part is a
point-to-point sum of r^{2n} with strengths scaled by log(h/h0) per source
box (``:4909-5016``, the default "p2p" mode).
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib

__all__ = ["series_terms", "remainder_coefficients", "remainder_series",
           "max_neighbor_distance", "split_scaling_codes", "split_correction",
           "split_term_keys", "split_extra_terms", "term_kernel", "term_scaling_code",
           "term_build_orders", "log_alpha_per_source", "radial_power_sum",
           "select_split_order_from_rho", "choose_auto_split_order", "split_rho_components"]

_GAMMA = 0.5772156649015329   # Euler-Mascheroni


def series_terms(dim, k, r_max, tol=1.0e-16, max_n=96):
    """Number of series terms for |k| r <= |k| r_max."""
    z = abs(complex(k)) * float(r_max)
    if dim == 3:
        if z == 0.0:
            return 1
        mag, n = z, 1
        while n < max_n and mag > tol:
            n += 1
            mag *= z / n
        return min(max_n, n + 2)
    if dim != 2:
        raise NotImplementedError("split remainder series supports only 2D/3D")
    if z == 0.0:
        return 1
    q = 0.25 * z * z
    mag, n = q, 1
    scale = max(1.0, abs(math.log(max(r_max, 1.0e-300))),
                abs(math.log(max(0.5 * abs(complex(k)), 1.0e-300))) + _GAMMA)
    while n < max_n and mag * scale > tol:
        n += 1
        mag *= q / (n * n)
    return min(max_n, n + 2)


def remainder_coefficients(dim, k, n_terms, split_order=1):
    """Coefficient array [2, n_terms + 1, 2] of ``vl1_split_correction``;
    split order p > 1 leaves out the terms the extra tables carry (2D the
    log terms of n < p, 3D the even n <= 2 (p - 1))."""
    k = complex(k)
    split_order = int(split_order)
    if split_order < 1:
        raise ValueError("split_order must be >= 1")
    out = np.zeros((2, n_terms + 1), dtype=np.complex128)
    if dim == 2:
        if k == 0:
            return np.zeros((2, n_terms + 1, 2))
        lk = np.log(0.5 * k) + _GAMMA
        out[0, 0] = 0.25j - lk / (2 * np.pi)
        harmonic = 0.0
        for n in range(1, n_terms + 1):
            harmonic += 1.0 / n
            s_n = ((-1) ** n) * (k * k / 4.0) ** n / (math.factorial(n) ** 2)
            if n >= split_order:
                out[0, n] = -s_n / (2 * np.pi)
            out[1, n] = s_n * ((harmonic - lk) / (2 * np.pi) + 0.25j)
    else:
        extracted = 2 * (split_order - 1)
        for n in range(1, n_terms + 1):
            if n % 2 == 0 and n <= extracted:
                continue
            out[0, n] = (1j * k) ** n / (4 * np.pi * math.factorial(n))
    return np.ascontiguousarray(np.stack([out.real, out.imag], axis=-1))


def split_term_keys(dim, split_order):
    """The extra term tables split order p needs (``expansion_wrangler_fpnd.py:
    4552-4570``): 2D ("power_log", 2n) for n = 1..p-1, 3D ("power", 2j - 1)
    for j = 1..p-1."""
    split_order = int(split_order)
    if dim == 2:
        return [("power_log", 2 * n) for n in range(1, split_order)]
    if dim == 3:
        return [("power", 2 * j - 1) for j in range(1, split_order)]
    raise NotImplementedError("helmholtz split extra terms are implemented only for 2D/3D")


def split_extra_terms(dim, k, split_order):
    """[(term key, coefficient)] of split order p
    (``expansion_wrangler_fpnd.py:5052-5115``): 2D a_n = -s_n / (2 pi) of
    r^{2n} log r, 3D c_{2j} = (i k)^{2j} / (4 pi (2j)!) of r^{2j-1}."""
    k = complex(k)
    out = []
    for key in split_term_keys(dim, split_order):
        if dim == 2:
            n = key[1] // 2
            s_n = ((-1) ** n) * (k * k / 4.0) ** n / (math.factorial(n) ** 2)
            out.append((key, complex(-s_n / (2 * np.pi))))
        else:
            n = key[1] + 1
            out.append((key, complex((1j * k) ** n / (4 * np.pi * math.factorial(n)))))
    return out


def term_kernel(dim, key):
    """The kernel of a term key: r^p or r^p log r."""
    from .kernels import RadialPowerKernel, RadialPowerLogKernel

    kind, power = key
    if kind == "power":
        return RadialPowerKernel(dim, power)
    if kind == "power_log":
        return RadialPowerLogKernel(dim, power)
    raise ValueError(f"unsupported split term kind {kind!r}")


def term_scaling_code(dim, power):
    """Single-table scaling of a term table, (h / h0)^(dim + power)
    (``expansion_wrangler_fpnd.py:4777-4799``, no derivatives)."""
    e = int(dim) + int(power)
    if e == 0:
        return "1.0"
    return ("(" + " * ".join(["BOX_extent"] * e) + ") / ("
            + " * ".join(["table_root_extent"] * e) + ")")


def term_build_orders(dim, q):
    """Default Duffy orders of the term tables (regular, radial)
    (``expansion_wrangler_fpnd.py:4596-4619``)."""
    if dim == 2:
        return max(8, 4 * q), max(21, 10 * q)
    return (6, 21) if q <= 2 else (8, 31)


def log_alpha_per_source(tree, table_root_extent):
    """log(box extent / table_root_extent) for each source point, by its
    box (``expansion_wrangler_fpnd.py:4909-4974``)."""
    h0 = float(table_root_extent)
    if h0 <= 0.0:
        raise ValueError("table_root_extent must be positive")
    starts = np.asarray(tree.box_source_starts, dtype=np.int64)
    counts = np.asarray(tree.box_source_counts_nonchild, dtype=np.int64)
    levels = np.asarray(tree.box_levels, dtype=np.int64)[: len(counts)]
    n = int(np.max(starts + counts)) if starts.size else 0
    beta = np.zeros(n, dtype=np.float64)
    root = float(tree.root_extent)
    for b in np.nonzero(counts > 0)[0]:
        beta[starts[b]:starts[b] + counts[b]] = np.log(root * 0.5 ** int(levels[b]) / h0)
    return beta


def select_split_order_from_rho(rho, thresholds, orders):
    """The order of the first threshold rho does not exceed, else the last
    order (``expansion_wrangler_fpnd.py:385-393``)."""
    if len(orders) != len(thresholds) + 1:
        raise ValueError("orders must have one more element than thresholds")
    for i, t in enumerate(thresholds):
        if float(rho) <= float(t):
            return int(orders[i])
    return int(orders[-1])


def split_rho_components(tree, wave_numbers):
    """(|Re k| h_max, |Im k| h_max) over the wave numbers, h_max the extent
    of the coarsest box holding sources (``expansion_wrangler_fpnd.py:
    4213-4250``)."""
    ks = [complex(k) for k in wave_numbers]
    counts = np.asarray(tree.box_source_counts_nonchild)
    levels = np.asarray(tree.box_levels)[: len(counts)]
    active = levels[counts > 0]
    if not ks or active.size == 0:
        return 0.0, 0.0
    h_max = float(tree.root_extent) * 0.5 ** int(active.min())
    return (max(abs(k.real) for k in ks) * h_max, max(abs(k.imag) for k in ks) * h_max)


def choose_auto_split_order(auto_cfg, rho_real, rho_imag):
    """Split order for rho = |k| h_max (``expansion_wrangler_fpnd.py:
    4252-4323``): thresholds and orders from ``auto_cfg`` ("rho_thresholds",
    "orders", "rho_thresholds_real" / "_imag") or geometric ladders
    rho_base * 2^j (real 0.25, imaginary 0.5 by default) over orders
    order_min (2) .. order_max (12); the larger of the real and imaginary
    parts' orders, clamped to [order_min, order_max] unless orders are
    given.  Returns (order, info)."""
    order_min = int(auto_cfg.get("order_min", 2))
    order_max = int(auto_cfg.get("order_max", 12))
    if order_max < order_min:
        raise ValueError("order_max must be >= order_min")
    if "rho_thresholds" in auto_cfg or "orders" in auto_cfg:
        t_real = tuple(auto_cfg.get("rho_thresholds", (0.5, 1.5, 3.0)))
        t_imag = t_real
        orders = (tuple(auto_cfg["orders"]) if "orders" in auto_cfg
                  else tuple(range(order_min, order_min + len(t_real) + 1)))
    else:
        r0, i0 = float(auto_cfg.get("rho_base_real", 0.25)), float(
            auto_cfg.get("rho_base_imag", 0.5))
        if r0 <= 0.0 or i0 <= 0.0:
            raise ValueError("rho_base_real and rho_base_imag must be positive")
        count = max(0, order_max - order_min)
        t_real = tuple(r0 * 2.0 ** j for j in range(count))
        t_imag = tuple(i0 * 2.0 ** j for j in range(count))
        orders = tuple(range(order_min, order_max + 1))
    if "rho_thresholds_real" in auto_cfg:
        t_real = tuple(auto_cfg["rho_thresholds_real"])
    if "rho_thresholds_imag" in auto_cfg:
        t_imag = tuple(auto_cfg["rho_thresholds_imag"])
    if "orders" not in auto_cfg:
        if len(t_real) != len(t_imag):
            raise ValueError("rho_thresholds_real and rho_thresholds_imag must have the "
                             "same length when orders are not provided")
        orders = tuple(range(order_min, order_min + len(t_real) + 1))
    order = max(select_split_order_from_rho(rho_real, t_real, orders),
                select_split_order_from_rho(rho_imag, t_imag, orders))
    if "orders" not in auto_cfg:
        order = max(order_min, min(order_max, order))
    coverage = max(float(t_real[-1]) if t_real else 0.0, float(t_imag[-1]) if t_imag else 0.0)
    return order, {"rho_real": float(rho_real), "rho_imag": float(rho_imag),
                   "thresholds_real": t_real, "thresholds_imag": t_imag, "orders": orders,
                   "beyond_coverage": bool(coverage > 0.0 and
                                           max(rho_real, rho_imag) > coverage)}


def remainder_series(dim, k, r, n_terms, split_order=1):
    """R(r) from the truncated series (numpy, for checks)."""
    c = remainder_coefficients(dim, k, n_terms, split_order)
    c = c[..., 0] + 1j * c[..., 1]
    r = np.asarray(r, dtype=np.float64)
    if dim == 2:
        x = r * r
        with np.errstate(divide="ignore"):
            lg = np.where(r > 1e-300, np.log(np.maximum(r, 1e-300)), 0.0)
        out = np.full(r.shape, c[0, 0])
        for n in range(1, n_terms + 1):
            out = out + (c[0, n] * lg + c[1, n]) * x ** n
        return out
    out = np.zeros(r.shape, dtype=np.complex128)
    for n in range(1, n_terms + 1):
        out = out + c[0, n] * r ** (n - 1)
    return out


def max_neighbor_distance(tree):
    """2 sqrt(dim) times the extent of the coarsest box holding sources
    (``expansion_wrangler_fpnd.py:4325-4335``)."""
    counts = np.asarray(tree.box_source_counts_nonchild)
    levels = np.asarray(tree.box_levels)[: len(counts)]
    active = levels[counts > 0]
    if active.size == 0:
        return 0.0
    return float(2.0 * np.sqrt(tree.dimensions) * tree.root_extent * 0.5 ** int(active.min()))


def split_scaling_codes(dim):
    """list-1 kernel scaling and displacement codes of the split mode's
    Laplace-table part (``expansion_wrangler_fpnd.py:4801-4833``, no
    derivatives): scaling (h / h_0)^2 in 2D and 3D; the 2D log
    displacement."""
    scaling = "(sbox_extent * sbox_extent) / (table_root_extent * table_root_extent)"
    if dim == 2:
        disp = (f"-0.5 / {np.pi!r} * scaling * log(sbox_extent / table_root_extent) * "
                "mode_nmlz[table_lev, sid]")
    else:
        disp = "0.0"
    return scaling, disp


def split_correction(tree_view, points, weights, k, n_terms, *, exclude_self=True,
                     stream=None, split_order=1):
    """The list-1 remainder sum on the GPU.

    ``tree_view``: a ``vl1_tree_view`` (device arrays); ``points``: CUDA
    float64 [dim, N] (tree order); ``weights``: CUDA float64 or complex128 [N]
    (density x quadrature weight).  Returns CUDA complex128 [N] (zero for
    points outside the target boxes)."""
    dim = int(points.shape[0])
    coef = remainder_coefficients(dim, k, n_terms, split_order)
    # a real wave number: the kernel's two-sum form of the series (in 2D it
    # needs every log term, i.e. split order 1)
    real_k = complex(k).imag == 0.0 and (dim == 3 or int(split_order) == 1)
    return _series_sum(tree_view, points, weights, coef, n_terms, exclude_self,
                       _lib.VL1_SPLIT_REAL_K if real_k else 0, stream)


def radial_power_sum(tree_view, points, weights, power, *, exclude_self=True, stream=None):
    """sum over list-1 source points of weights x r^power on the GPU (the
    series kernel with one coefficient; 2D: even powers)."""
    dim = int(points.shape[0])
    power = int(power)
    if dim == 2:
        if power < 2 or power % 2:
            raise ValueError("2D radial power sums take even powers >= 2")
        n_terms = power // 2
        coef = np.zeros((2, n_terms + 1, 2))
        coef[1, n_terms, 0] = 1.0
    else:
        if power < 0:
            raise ValueError("power must be non-negative")
        n_terms = power + 1
        coef = np.zeros((2, n_terms + 1, 2))
        coef[0, n_terms, 0] = 1.0
    return _series_sum(tree_view, points, weights, coef, n_terms, exclude_self, 0, stream)


def _series_sum(tree_view, points, weights, coef_np, n_terms, exclude_self, flags, stream):
    import torch

    dim = int(points.shape[0])
    n = int(points.shape[1])
    if weights.numel() != n:
        raise ValueError("weights must have one value per point")
    w = weights.contiguous()
    wcplx = w.is_complex()
    if wcplx:
        w = torch.view_as_real(w.to(torch.complex128)).contiguous()
    else:
        w = w.to(torch.float64)
    coef = torch.from_numpy(np.ascontiguousarray(coef_np)).to("cuda")
    out = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    d = _lib.SplitDesc()
    d.dim, d.n_points, d.n_terms = dim, n, int(n_terms)
    d.exclude_self, d.weights_complex = int(bool(exclude_self)), int(wcplx)
    d.flags = int(flags)
    d.tree = C.cast(C.pointer(tree_view), C.c_void_p)
    pts = points.to(torch.float64).contiguous()
    d.points, d.weights = pts.data_ptr(), w.data_ptr()
    d.coefficients, d.result = coef.data_ptr(), out.data_ptr()
    sh = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.lib().vl1_split_correction(C.byref(d), C.c_void_p(sh)),
               "vl1_split_correction")
    return torch.view_as_complex(out)
