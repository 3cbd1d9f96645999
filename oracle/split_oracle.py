"""CPU restatement of the Helmholtz split correction (numpy, FP64).

TEST INFRASTRUCTURE.  Only ``tests/`` imports this module.  It sums, per
target point, (density x weight) x (G_k - G_0)(r) over the points of the
target box's list-1 source boxes (``volumential/expansion_wrangler_fpnd.py:
3491-3836``, self pairs excluded when asked), with the remainder in closed
form instead of the product's series: 2D
(i/4) H0^(1)(k r) + log(r) / (2 pi), tending to i/4 - (log(k/2) + gamma)/(2 pi)
at r = 0; 3D (exp(i k r) - 1) / (4 pi r) via expm1, tending to i k / (4 pi).
Split order p > 1 (``:212-332, 5052-5115``) subtracts the extracted terms in
closed form: 2D a_n r^{2n} log r (n < p, a_n = (-1)^(n+1) (k^2/4)^n /
((n!)^2 2 pi)), 3D (i k)^{2j} r^{2j-1} / (4 pi (2j)!) (j < p).
"""

from __future__ import annotations

import math

import numpy as np
from scipy import special


def extracted_terms(dim, k, split_order):
    """[(kind, power, coefficient)] of the terms split order p moves into
    tables."""
    k = complex(k)
    out = []
    for n in range(1, int(split_order)):
        if dim == 2:
            a = -((-1) ** n) * (k * k / 4.0) ** n / (math.factorial(n) ** 2 * 2 * np.pi)
            out.append(("power_log", 2 * n, a))
        else:
            out.append(("power", 2 * n - 1, (1j * k) ** (2 * n) /
                        (4 * np.pi * math.factorial(2 * n))))
    return out


def radial_term(kind, power, r):
    r = np.asarray(r, dtype=np.float64)
    if kind == "power":
        return r ** power
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(r > 0, r ** power * np.log(np.where(r > 0, r, 1.0)), 0.0)


def remainder(dim, k, r, split_order=1):
    r = np.asarray(r, dtype=np.float64)
    out = _remainder1(dim, k, r)
    for kind, power, c in extracted_terms(dim, k, split_order):
        out = out - c * radial_term(kind, power, r)
    return out


def _remainder1(dim, k, r):
    k = complex(k)
    if dim == 2:
        with np.errstate(divide="ignore", invalid="ignore"):
            v = 0.25j * special.hankel1(0, k * r) + np.log(r) / (2 * np.pi)
        lim = 0.25j - (np.log(0.5 * k) + np.euler_gamma) / (2 * np.pi)
        return np.where(r > 0, v, lim)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.expm1(1j * k * r) / (4 * np.pi * r)
    return np.where(r > 0, v, 1j * k / (4 * np.pi))


def log_alpha(box_levels, box_starts, box_counts, root_extent, table_root_extent):
    """Per point log(h / h0) of its box (``expansion_wrangler_fpnd.py:
    4909-4974``)."""
    n = int(np.max(np.asarray(box_starts) + np.asarray(box_counts)))
    out = np.zeros(n)
    for b in range(len(box_counts)):
        if box_counts[b] > 0:
            h = root_extent * 0.5 ** int(box_levels[b])
            out[box_starts[b]:box_starts[b] + box_counts[b]] = np.log(h / table_root_extent)
    return out


def split_sum(dim, k, points, weights, target_boxes, starts, lists, box_starts, box_counts,
              exclude_self=True, split_order=1, kernel=None):
    """``kernel(r)`` replaces the remainder when given (a radial power)."""
    n = points.shape[1]
    out = np.zeros(n, dtype=np.complex128)
    for i, tb in enumerate(target_boxes):
        tgt = np.arange(box_starts[tb], box_starts[tb] + box_counts[tb])
        src = np.concatenate([np.arange(box_starts[sb], box_starts[sb] + box_counts[sb])
                              for sb in lists[starts[i]:starts[i + 1]]])
        d = points[:, tgt][:, :, None] - points[:, src][:, None, :]
        r = np.sqrt(np.sum(d * d, axis=0))
        g = remainder(dim, k, r, split_order) if kernel is None else kernel(r)
        if exclude_self:
            g = np.where(tgt[:, None] == src[None, :], 0.0, g)
        out[tgt] = g @ weights[src]
    return out
