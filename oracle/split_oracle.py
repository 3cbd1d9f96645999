"""CPU restatement of the Helmholtz split correction (numpy, FP64).

TEST INFRASTRUCTURE.  Only ``tests/`` imports this module.  It sums, per
target point, (density x weight) x (G_k - G_0)(r) over the points of the
target box's list-1 source boxes (``volumential/expansion_wrangler_fpnd.py:
3491-3836``, split order 1, self pairs excluded when asked), with the
remainder in closed form instead of the product's series: 2D
(i/4) H0^(1)(k r) + log(r) / (2 pi), tending to i/4 - (log(k/2) + gamma)/(2 pi)
at r = 0; 3D (exp(i k r) - 1) / (4 pi r) via expm1, tending to i k / (4 pi).
"""

from __future__ import annotations

import numpy as np
from scipy import special


def remainder(dim, k, r):
    r = np.asarray(r, dtype=np.float64)
    k = complex(k)
    if dim == 2:
        with np.errstate(divide="ignore", invalid="ignore"):
            v = 0.25j * special.hankel1(0, k * r) + np.log(r) / (2 * np.pi)
        lim = 0.25j - (np.log(0.5 * k) + np.euler_gamma) / (2 * np.pi)
        return np.where(r > 0, v, lim)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.expm1(1j * k * r) / (4 * np.pi * r)
    return np.where(r > 0, v, 1j * k / (4 * np.pi))


def split_sum(dim, k, points, weights, target_boxes, starts, lists, box_starts, box_counts,
              exclude_self=True):
    n = points.shape[1]
    out = np.zeros(n, dtype=np.complex128)
    for i, tb in enumerate(target_boxes):
        tgt = np.arange(box_starts[tb], box_starts[tb] + box_counts[tb])
        src = np.concatenate([np.arange(box_starts[sb], box_starts[sb] + box_counts[sb])
                              for sb in lists[starts[i]:starts[i + 1]]])
        d = points[:, tgt][:, :, None] - points[:, src][:, None, :]
        r = np.sqrt(np.sum(d * d, axis=0))
        g = remainder(dim, k, r)
        if exclude_self:
            g = np.where(tgt[:, None] == src[None, :], 0.0, g)
        out[tgt] = g @ weights[src]
    return out
