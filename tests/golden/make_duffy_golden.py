"""Golden vectors of the Duffy radial table builder, from the reference itself.

Run where the reference source tree is mounted (read only):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_duffy_golden.py /path/to/reference

Imports by file path only numpy/scipy/mpmath modules of the reference:
``volumential/singular_integral_2d.py`` (the 1D rules
``_duffy_radial_nodes_weights`` / ``_duffy_regular_nodes_weights`` and the
scalar Duffy integrator ``box_quad_duffy_radial_nd``, which runs the same node
scheme as the batched builder), ``volumential/lagrange.py`` (the source modes'
barycentric Lagrange basis) and ``volumential/list1_gallery.py`` (case
vectors).  The target point of a case follows ``find_target_point``
(``volumential/nearfield_potential_table.py:917-946``) and the source mode
``get_mode`` (``:749-800``).  The kernels are the standard free-space Green's
functions with their scaling constants (sumpy, which the reference takes them
from, is not available).

Output: ``duffy_golden.npz`` with the 1D rules and a set of table entries
(dim, q, kernel, k, case, source mode, target point, orders, value).
"""

from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np
from scipy import special

HERE = os.path.dirname(os.path.abspath(__file__))
sys.dont_write_bytecode = True

KERNELS = {"laplace": 0, "helmholtz": 1}


def load_ref(ref_root, name):
    path = os.path.join(ref_root, "volumential", f"{name}.py")
    spec = importlib.util.spec_from_file_location(f"_ref_{name}", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def green(kind, dim, k, *d):
    r = np.sqrt(sum(x * x for x in d))
    if kind == "laplace":
        return -np.log(r) / (2 * np.pi) if dim == 2 else 1.0 / (4 * np.pi * r)
    if dim == 2:
        return 0.25j * (special.j0(k * r) + 1j * special.y0(k * r))
    return np.exp(1j * k * r) / (4 * np.pi * r)


def main():
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the volumential source tree>")
    ref = sys.argv[1]
    sq = load_ref(ref, "singular_integral_2d")
    lg = load_ref(ref, "lagrange")
    gal = load_ref(ref, "list1_gallery")
    out = {}
    for n in (11, 21, 31, 61):
        x, w = sq._duffy_radial_nodes_weights("tanh-sinh-fast", n, 50)
        out[f"radial_fast_{n}_x"], out[f"radial_fast_{n}_w"] = x, w
    for dm1 in (1, 2):
        for order in (4, 6, 8):
            x, w = sq._duffy_regular_nodes_weights(dm1, order)
            out[f"regular_{dm1}_{order}_x"] = np.asarray(x)
            out[f"regular_{dm1}_{order}_w"] = np.asarray(w)

    rows = []
    rng = np.random.default_rng(7)
    extent = 1.0
    for dim, qs, reg, rad, n_rand in ((2, (1, 2, 3), 6, 21, 4), (3, (1, 2), 4, 11, 1)):
        vecs = gal.generate_list1_gallery(dim)[0]
        mags = [int(np.max(np.abs(v))) for v in vecs]
        picks = []
        for m in sorted(set(mags)):
            picks.append(mags.index(m))          # one case of every size class
        picks += list(rng.choice(len(vecs), size=n_rand, replace=False))
        for q in qs:
            gx, _ = np.polynomial.legendre.leggauss(q)
            xi = 0.5 * extent * (gx + 1.0)
            bw = lg.barycentric_lagrange_weights(xi)
            nq = q ** dim
            for kind in ("laplace", "helmholtz"):
                k = 0.0 if kind == "laplace" else 3.0
                for case in picks:
                    smode = int(rng.integers(nq))
                    tpoint = int(rng.integers(nq))
                    sidx = np.unravel_index(smode, (q,) * dim)
                    tidx = np.unravel_index(tpoint, (q,) * dim)
                    vec = np.asarray(vecs[case], dtype=np.float64)
                    center = np.full(dim, 0.5 * extent) + vec / 4.0 * extent
                    m = int(np.max(np.abs(vec)))
                    size = 1.0 if m == 0 else (m - 2.0) / 2.0
                    target = center + size * (np.array([xi[i] for i in tidx]) - 0.5 * extent)

                    def integrand(*y, target=target, sidx=sidx, q=q, xi=xi, bw=bw, k=k,
                                  kind=kind, dim=dim):
                        mode = 1.0
                        if q > 1:
                            for a in range(dim):
                                mode *= lg.evaluate_lagrange_basis_1d(xi, sidx[a], y[a],
                                                                      weights=bw)
                        return mode * green(kind, dim, k,
                                            *[target[a] - y[a] for a in range(dim)])

                    val, _ = sq.box_quad_duffy_radial_nd(
                        integrand, [(0.0, extent)] * dim, tuple(target),
                        radial_rule="tanh-sinh-fast", deg_regular=reg,
                        radial_quad_order=rad)
                    rows.append((dim, q, KERNELS[kind], k, case, smode, tpoint, reg, rad,
                                 complex(val)))
    a = np.array(rows, dtype=object)
    out["entry_ints"] = np.array([[r[0], r[1], r[2], r[4], r[5], r[6], r[7], r[8]]
                                  for r in rows], dtype=np.int64)
    out["entry_k"] = np.array([r[3] for r in rows])
    out["entry_value"] = np.array([r[9] for r in rows], dtype=np.complex128)
    np.savez_compressed(os.path.join(HERE, "duffy_golden.npz"), **out)
    print(f"{len(a)} entries")


if __name__ == "__main__":
    main()
