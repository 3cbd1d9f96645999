"""CPU restatement of the Duffy radial table builder (numpy, FP64).

TEST INFRASTRUCTURE.  Only ``tests/`` imports this module; the product
package never does.  It evaluates table entries with the node set of the
reference's batched builder, enumerated explicitly in the reference's loop
order (``volumential/nearfield_potential_table.py:2225-2291``: sign vectors
x axis permutations x tail nodes x radial nodes), and the integrand of
``:2035-2223`` (sub-box lengths from the target clipped into the box, the
Duffy map, the second-form barycentric Lagrange basis of ``:2113-2124`` with
its node-hit rule, nodes on the singular point dropped).  The 1D rules are the
reference's (``volumential/singular_integral_2d.py:807-853``), restated here
independently of the product's ``table_builder``; both are pinned to rules
generated by the reference itself (``tests/golden/duffy_golden.npz``).

Kernels are the standard free-space Green's functions with their scaling
constants (the reference takes them from sumpy, absent here).
"""

from __future__ import annotations

from itertools import permutations, product

import numpy as np
from scipy import special

__all__ = ["tanh_sinh_fast", "gauss_legendre_tail", "node_set", "green", "entry_values",
           "target_point"]


def tanh_sinh_fast(order):
    n = max(3, int(order))
    h = 1.0 / np.sqrt(n)
    t = h * np.arange(-n, n + 1, dtype=np.float64)
    arg = 0.5 * np.pi * np.sinh(t)
    x = 0.5 * (1.0 + np.tanh(arg))
    ex = np.exp(-2.0 * np.abs(arg))
    w = 0.25 * np.pi * h * np.cosh(t) * 4.0 * ex / (1.0 + ex) ** 2
    keep = (x > 0.0) & (x < 1.0) & np.isfinite(w)
    return x[keep], w[keep]


def gauss_legendre_tail(dim_minus_one, order):
    if dim_minus_one == 0:
        return np.zeros((1, 0)), np.ones(1)
    x, w = special.roots_legendre(order)
    x, w = 0.5 * (x + 1.0), 0.5 * w
    g = np.meshgrid(*([x] * dim_minus_one), indexing="ij")
    gw = np.meshgrid(*([w] * dim_minus_one), indexing="ij")
    return np.stack([a.ravel() for a in g], axis=-1), np.prod(np.array(gw), axis=0).ravel()


def node_set(dim, regular_order, radial_order):
    """(u [dim, n], sign [dim, n], jac_base [n]) in the reference's order."""
    tail_x, tail_w = gauss_legendre_tail(dim - 1, regular_order)
    rho, w_rho = tanh_sinh_fast(radial_order)
    us, sgs, jacs = [], [], []
    for signs in product([-1.0, 1.0], repeat=dim):
        for perm in permutations(range(dim)):
            for ireg in range(len(tail_w)):
                for r, wr in zip(rho, w_rho):
                    rs = np.concatenate([[r], tail_x[ireg]])
                    u = np.empty(dim)
                    cum = 1.0
                    for i, axis in enumerate(perm):
                        cum *= rs[i]
                        u[axis] = cum
                    jac = 1.0
                    for i in range(dim - 1):
                        jac *= rs[i] ** (dim - 1 - i)
                    us.append(u)
                    sgs.append(signs)
                    jacs.append(jac * tail_w[ireg] * wr)
    return np.array(us).T, np.array(sgs).T, np.array(jacs)


def green(kind, dvec, k=0.0, power=0, derivative=0):
    """Kernel value times scaling constant at displacements dvec [dim, n]
    ("power" r^p and "power_log" r^p log r: the split-term kernels of
    ``volumential/expansion_wrangler_fpnd.py:144-209``, constant 1).
    ``derivative`` a + 1: d/dt_a, -(a + 1): d/dy_a (Laplace, Helmholtz)."""
    r = np.sqrt(np.sum(dvec * dvec, axis=0))
    if derivative:
        a = abs(derivative) - 1
        sgn = 1.0 if derivative > 0 else -1.0
        da = dvec[a]
        dim = dvec.shape[0]
        if kind == "laplace":
            g = -da / (2 * np.pi * r * r) if dim == 2 else -da / (4 * np.pi * r ** 3)
        elif kind == "helmholtz":
            if dim == 2:
                g = -0.25j * k * special.hankel1(1, k * r) * da / r
            else:
                g = np.exp(1j * k * r) * (1j * k * r - 1.0) * da / (4 * np.pi * r ** 3)
        else:
            raise ValueError(f"no derivative of the {kind} kernel")
        return sgn * g
    if kind == "power":
        return r ** power
    if kind == "power_log":
        return r ** power * np.log(r)
    if kind == "laplace":
        return -np.log(r) / (2 * np.pi) if dvec.shape[0] == 2 else 1.0 / (4 * np.pi * r)
    if kind == "helmholtz":
        if dvec.shape[0] == 2:
            return 0.25j * (special.j0(k * r) + 1j * special.y0(k * r))
        return np.exp(1j * k * r) / (4 * np.pi * r)
    if kind == "constant":
        return np.ones_like(r)
    if kind == "plane_wave":
        return np.cos(k * dvec[0])
    raise ValueError(kind)


def target_point(dim, q, extent, case_vec, tpoint):
    """The case's target point (``nearfield_potential_table.py:917-946``)."""
    x, _ = np.polynomial.legendre.leggauss(q)
    nodes = 0.5 * extent * (x + 1.0)
    idx = np.unravel_index(tpoint, (q,) * dim)
    pt = np.array([nodes[i] for i in idx])
    vec = np.asarray(case_vec, dtype=np.float64)
    center = np.full(dim, 0.5 * extent) + vec / 4.0 * extent
    m = int(np.max(np.abs(vec)))
    size = 1.0 if m == 0 else (m - 2.0) / 2.0
    return center + size * (pt - 0.5 * extent)


def _basis(xi, bw, m, y, extent):
    """Second-form barycentric basis of node m at points y (the reference's
    rule: a point within 8 eps * extent of a node takes that node's value)."""
    tol = 8 * np.finfo(np.float64).eps * extent
    diff = y[None, :] - xi[:, None]
    hit = np.abs(diff) < tol
    safe = np.where(hit, 1.0, diff)
    terms = np.where(hit, 0.0, bw[:, None] / safe)
    den = terms.sum(axis=0)
    num = np.where(hit[m], 0.0, bw[m] / safe[m])
    any_hit = hit.any(axis=0)
    return np.where(any_hit, hit[m].astype(np.float64), num / np.where(den == 0, 1, den))


def entry_values(dim, q, extent, kind, targets, modes, regular_order, radial_order, k=0.0,
                 power=0, derivative=0):
    """Table values of entries with target points ``targets`` [dim, n] and
    source mode axes ``modes`` [dim, n]."""
    u, sg, jac = node_set(dim, regular_order, radial_order)
    x, _ = np.polynomial.legendre.leggauss(q)
    xi = 0.5 * extent * (x + 1.0)
    d = xi[:, None] - xi[None, :]
    np.fill_diagonal(d, 1.0)
    bw = 1.0 / np.prod(d, axis=1)
    out = []
    for e in range(targets.shape[1]):
        t = targets[:, e]
        dc = np.clip(t, 0.0, extent)
        lens = np.where(sg < 0, dc[:, None], extent - dc[:, None])
        active = np.all(lens > 0, axis=0)
        y = dc[:, None] + sg * lens * u
        dv = t[:, None] - y
        r2 = np.sum(dv * dv, axis=0)
        active &= r2 > 0
        w = jac * np.prod(lens, axis=0)
        basis = np.ones(u.shape[1])
        if q > 1:
            for a in range(dim):
                basis *= _basis(xi, bw, int(modes[a, e]), y[a], extent)
        with np.errstate(divide="ignore", invalid="ignore"):
            g = green(kind, np.where(active[None, :], dv, 1.0), k, power, derivative)
        out.append(np.sum(np.where(active, g * w * basis, 0.0)))
    return np.array(out)
