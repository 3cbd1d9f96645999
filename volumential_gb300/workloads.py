"""Seeded synthetic workloads of the list-1 benchmark configurations.

The reference measures nothing on a public dataset; its benchmark shapes are
stated as configurations (uniform/adaptive quadtrees and octrees on
``[-0.5, 0.5]^dim`` with tensor Gauss-Legendre nodes, densities that are sums
of Gaussians ``a * exp(-|x - c|^2 / w^2)`` with seeded centres, log-uniform
widths and N(0, 1) amplitudes).  This module builds them with
``numpy.random.default_rng(seed)``.

Table values.  ``duffy_tables`` builds the tables the configurations name
(Laplace, Helmholtz) with the package's FP64 GPU Duffy builder at the
reference's default orders (regular 20, radial 61, tanh-sinh-fast;
``nearfield_potential_table.py:2948-2953``); C1, C2 and C3 use them by default.
``synthetic_tables`` fills the compact (orbit-reduced) layout with seeded
N(0, 0.1) values instead: it needs no GPU and serves the host-side tests and
the parity tests of the index arithmetic, which do not depend on the values.
The mixed-precision path's error does depend on them (each table value is
held to 2^-40 of the table's largest one), which is why the headline
configurations run on the physical tables.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .kernels import ConstantKernel, HelmholtzKernel, LaplaceKernel
from .nearfield_potential_table import NearFieldInteractionTable
from .tree_build import (
    Traversal,
    build_adaptive_tree,
    build_list1_traversal,
    build_uniform_tree,
)

__all__ = ["GaussianMixture", "random_gaussian_mixture", "synthetic_tables", "duffy_tables",
           "make_tables",
           "Workload", "config_c1", "config_c2", "config_c3", "uniform_workload",
           "adaptive_workload", "config_c4", "config_c5", "config_c5_arrivals",
           "c5_arrival_workloads", "C5Problem", "poisson_arrivals"]


@dataclass
class GaussianMixture:
    centers: np.ndarray   # [n_terms, dim]
    widths: np.ndarray    # [n_terms]
    amps: np.ndarray      # [n_terms]

    def __call__(self, points):
        """Density at ``points`` ([dim, ...]); returns [...]."""
        pts = np.asarray(points)
        out = np.zeros(pts.shape[1:])
        for c, w, a in zip(self.centers, self.widths, self.amps):
            d2 = np.zeros(pts.shape[1:])
            for ax in range(pts.shape[0]):
                d2 += (pts[ax] - c[ax]) ** 2
            out += a * np.exp(-d2 / (w * w))
        return out

    def on_device(self, points):
        """The same density evaluated with torch where ``points`` ([dim, N]
        float64 tensor) lives."""
        import torch

        out = torch.zeros(points.shape[1:], dtype=torch.float64, device=points.device)
        for c, w, a in zip(self.centers, self.widths, self.amps):
            d2 = torch.zeros_like(out)
            for ax in range(points.shape[0]):
                d2 += (points[ax] - float(c[ax])) ** 2
            out += float(a) * torch.exp(-d2 / float(w * w))
        return out


def random_gaussian_mixture(rng, dim, n_terms, width_range, a=-0.5, b=0.5):
    lo, hi = width_range
    return GaussianMixture(
        centers=rng.uniform(a, b, size=(n_terms, dim)),
        widths=np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_terms)),
        amps=rng.standard_normal(n_terms))


def synthetic_tables(dim, q, kernel, *, n_tables=1, seed=0, source_box_extent=1.0,
                     complex_values=False):
    """Tables with the reference's compact layout filled with seeded values.

    Level ``l`` has source box extent ``source_box_extent / 2**l``.
    """
    rng = np.random.default_rng(seed)
    out = []
    for lev in range(n_tables):
        t = NearFieldInteractionTable(
            q, dim=dim, sumpy_kernel=kernel,
            source_box_extent=source_box_extent * 0.5 ** lev,
            dtype=np.complex128 if complex_values else np.float64)
        info = t._get_scalar_arithmetic_invariant_entry_info()
        n = len(info["entry_ids"])
        vals = rng.standard_normal(n) * 0.1
        if complex_values:
            vals = vals + 1j * rng.standard_normal(n) * 0.1
        t.set_reduced_table_data(info["entry_ids"], vals)
        if dim == 2:
            t.build_normalizer_table()
        out.append(t)
    return out


#: (dim, q, kernel name, k, n_tables, extent, orders) -> built tables; a table
#: set is built once per process (the 3D q = 5 Laplace table takes ~2 s)
_DUFFY_CACHE: dict = {}


def duffy_tables(dim, q, kernel, *, n_tables=1, source_box_extent=1.0, k=None,
                 complex_values=False, regular_quad_order=20, radial_quad_order=61,
                 max_ctas=0):
    """Tables of ``kernel`` with values from the FP64 GPU Duffy builder.

    Level ``l`` has source box extent ``source_box_extent / 2**l``; Helmholtz
    needs the wave number ``k``.  Orders default to the reference's
    (``nearfield_potential_table.py:2948-2953``).  ``max_ctas`` > 0 caps the
    builder's grid (same values; a build beside other GPU work).  Needs a CUDA
    device."""
    kname = type(kernel).__name__
    key = (dim, q, kname, None if k is None else float(k), n_tables,
           float(source_box_extent), complex_values, regular_quad_order, radial_quad_order)
    hit = _DUFFY_CACHE.get(key)
    if hit is not None:
        return list(hit)
    out = []
    for lev in range(n_tables):
        t = NearFieldInteractionTable(
            q, dim=dim, sumpy_kernel=kernel,
            source_box_extent=source_box_extent * 0.5 ** lev,
            dtype=np.complex128 if complex_values else np.float64)
        kw = {} if k is None else {"k": float(k)}
        if max_ctas:
            kw["max_ctas"] = int(max_ctas)
        t.build_table_via_duffy_radial(regular_quad_order=regular_quad_order,
                                       radial_quad_order=radial_quad_order, **kw)
        out.append(t)
    _DUFFY_CACHE[key] = tuple(out)
    return out


def make_tables(source, dim, q, kernel, *, n_tables=1, seed=0, source_box_extent=1.0,
                complex_values=False, k=None, orders=None):
    """``source`` "duffy" (physical values, GPU builder) or "synthetic"
    (seeded values, no GPU)."""
    if source == "duffy":
        return duffy_tables(dim, q, kernel, n_tables=n_tables,
                            source_box_extent=source_box_extent, k=k,
                            complex_values=complex_values, **(orders or {}))
    if source == "synthetic":
        return synthetic_tables(dim, q, kernel, n_tables=n_tables, seed=seed,
                                source_box_extent=source_box_extent,
                                complex_values=complex_values)
    raise ValueError(f"table source must be 'duffy' or 'synthetic', got {source!r}")


@dataclass
class Workload:
    name: str
    dim: int
    q: int
    kernel: object
    traversal: Traversal
    tables: list
    coefs: np.ndarray            # [nrhs, N] (float64 or complex128)
    seed: int
    meta: dict = field(default_factory=dict)

    @property
    def tree(self):
        return self.traversal.tree

    @property
    def n_points(self):
        return self.tree.ntargets

    @property
    def nrhs(self):
        return int(self.coefs.shape[0])

    def pair_count(self):
        """P = sum over list-1 box pairs of n_target * n_source points."""
        tr = self.traversal
        counts = self.tree.box_target_counts_nonchild.astype(np.int64)
        nt = np.repeat(counts[tr.target_boxes], np.diff(tr.neighbor_source_boxes_starts))
        ns = counts[tr.neighbor_source_boxes_lists]
        return int(np.sum(nt * ns))


def _densities(rng, tree, nrhs, n_terms, width_range):
    cols = []
    mixes = []
    for _ in range(nrhs):
        k = int(rng.integers(n_terms[0], n_terms[1] + 1)) if isinstance(n_terms, tuple) \
            else int(n_terms)
        lo = float(np.min(tree.root_vertex))
        mix = random_gaussian_mixture(rng, tree.dim, k, width_range, a=lo,
                                      b=lo + float(tree.root_extent))
        mixes.append(mix)
        cols.append(mix(tree.targets))
    return np.stack(cols), mixes


def uniform_workload(name, dim, level, q, *, kernel=None, nrhs=1, seed=0,
                     n_terms=8, width_range=(0.02, 0.1), n_tables=1,
                     complex_table=False, tables="synthetic", k=None, orders=None,
                     a=-0.5, b=0.5):
    """Uniform tree of ``level`` on [a, b]^dim; ``tables`` "synthetic" or
    "duffy" (canonical tables at the root extent, ``n_tables`` levels)."""
    rng = np.random.default_rng(seed)
    tree = build_uniform_tree(dim, level, q, a=a, b=b)
    trav = build_list1_traversal(tree)
    kernel = kernel or LaplaceKernel(dim)
    coefs, mixes = _densities(rng, tree, nrhs, n_terms, width_range)
    tabs = make_tables(tables, dim, q, kernel, n_tables=n_tables, seed=seed + 17,
                       source_box_extent=tree.root_extent, complex_values=complex_table,
                       k=k, orders=orders)
    return Workload(name, dim, q, kernel, trav, tabs, coefs, seed,
                    meta={"level": level, "mixtures": mixes, "tables": tables})


def adaptive_workload(name, dim, q, *, tol, max_level, min_level=2, kernel=None,
                      nrhs=1, seed=0, n_terms=16, width_range=(0.01, 0.08),
                      max_leaves=None, tables="synthetic", orders=None):
    """Adaptive tree refined where the density's variation over a leaf's
    nodes (max - min) exceeds ``tol``, then 2:1 balanced."""
    rng = np.random.default_rng(seed)
    mix = random_gaussian_mixture(rng, dim, n_terms, width_range)

    def refine(nodes):
        v = mix(nodes)
        return (v.max(axis=-1) - v.min(axis=-1)) > tol

    tree = build_adaptive_tree(dim, q, refine, max_level=max_level, min_level=min_level,
                               max_leaves=max_leaves)
    trav = build_list1_traversal(tree)
    kernel = kernel or LaplaceKernel(dim)
    cols = [mix(tree.targets)]
    for _ in range(nrhs - 1):
        m = random_gaussian_mixture(rng, dim, n_terms, width_range)
        cols.append(m(tree.targets))
    tabs = make_tables(tables, dim, q, kernel, seed=seed + 17,
                       source_box_extent=tree.root_extent, orders=orders)
    return Workload(name, dim, q, kernel, trav, tabs, np.stack(cols), seed,
                    meta={"tol": tol, "max_level": max_level, "mixture": mix,
                          "tables": tables})


def config_c1(seed=1000, tables="duffy"):
    """2D Laplace, uniform level 5, q=4 (1024 leaves, 16,384 points), 1 RHS;
    canonical 2D Laplace table (level 0, root extent) built by Duffy
    quadrature in FP64, inferred scaling and the log displacement."""
    return uniform_workload("c1_lap2d_uniform_l5_q4", 2, 5, 4, seed=seed, n_terms=8,
                            width_range=(0.02, 0.1), tables=tables)


def config_c2(seed=2006, tol=1e-3, max_level=6, tables="duffy"):
    """3D Laplace, adaptive 2:1-balanced octree, q=4, 16 Gaussians (w in
    [0.01, 0.08]), refined where the leaf variation (max - min of the density
    at the leaf's 64 nodes) exceeds ``tol``, leaves on levels 3..6.  With the
    default seed: 23,087 leaves, 1,477,568 points, 565,335 list-1 box pairs,
    2.32e9 point pairs.  Canonical 3D Laplace table (FP64 Duffy build),
    scaling h_s^2 / h_0^2."""
    return adaptive_workload("c2_lap3d_adaptive_q4", 3, 4, tol=tol, max_level=max_level,
                             seed=seed, n_terms=16, width_range=(0.01, 0.08),
                             tables=tables)


def config_c3(seed=3000, nrhs=256, k=20.0, tables="duffy", level=6):
    """2D Helmholtz (k=20, fixed single complex table at the tree's level),
    uniform level 6, q=5 (102,400 points), ``nrhs`` Gaussian-sum densities.
    The table is the Helmholtz kernel's, built by Duffy quadrature in FP64 at
    source box extent root / 2^level (``fixed_single_table``,
    list1.py:406-420)."""
    w = uniform_workload(f"c3_helm2d_uniform_l{level}_q5", 2, level, 5, seed=seed,
                         nrhs=nrhs, n_terms=8, width_range=(0.02, 0.1),
                         kernel=HelmholtzKernel(2), complex_table=True)
    w.tables = make_tables(tables, 2, 5, w.kernel, seed=seed + 17,
                           source_box_extent=w.tree.root_extent / 2.0 ** level,
                           complex_values=True, k=k)
    w.meta["k"] = k
    w.meta["tables"] = tables
    return w


def config_c4(seed=4000, n_problems=64, levels=(3, 6), qs=(3, 4, 5), nrhs_range=(1, 32),
              terms=(4, 16), width_range=(0.01, 0.1), tables="duffy", device_lists=True):
    """Uneven batch: ``n_problems`` independent 3D Laplace problems on uniform
    octrees, level uniform in ``levels`` (inclusive), q uniform in ``qs``, rhs
    count uniform in ``nrhs_range``, each density a sum of ``terms`` Gaussians.

    The densities are not evaluated here (``coefs`` has shape [nrhs, 0]):
    the mixtures are in ``meta["mixtures"]`` and are evaluated on the device
    (``GaussianMixture.on_device``).  Problems of one q share one table set
    (3D Laplace, FP64 Duffy build unless ``tables="synthetic"``) and problems
    of one (level, q) share one tree; ``device_lists`` builds the list-1 CSR
    on the GPU (a level-6 octree takes ~4 s on the host).
    """
    from .tree_build import build_list1_traversal_device

    rng = np.random.default_rng(seed)
    kernel = LaplaceKernel(3)
    table_sets = {}
    trees = {}
    out = []
    for i in range(n_problems):
        lev = int(rng.integers(levels[0], levels[1] + 1))
        q = int(rng.choice(qs))
        nrhs = int(rng.integers(nrhs_range[0], nrhs_range[1] + 1))
        if (lev, q) not in trees:
            tree = build_uniform_tree(3, lev, q)
            trees[(lev, q)] = (build_list1_traversal_device(tree) if device_lists
                               else build_list1_traversal(tree))
        trav = trees[(lev, q)]
        mixes = [random_gaussian_mixture(rng, 3, int(rng.integers(terms[0], terms[1] + 1)),
                                         width_range) for _ in range(nrhs)]
        if q not in table_sets:
            table_sets[q] = make_tables(tables, 3, q, kernel, seed=seed + 17 + q,
                                        source_box_extent=trav.tree.root_extent)
        out.append(Workload(f"c4_p{i:02d}_l{lev}_q{q}", 3, q, kernel, trav, table_sets[q],
                            np.zeros((nrhs, 0)), seed,
                            meta={"level": lev, "mixtures": mixes, "table_key": q,
                                  "tree_key": (lev, q), "tables": tables}))
    return out


@dataclass
class C5Problem:
    """One resident problem of the serving mix: a uniform tree and a table
    set.  ``table_key`` is shared by the problems that use the same tables:
    (dim, "laplace", 0, q) for Laplace, (dim, "helmholtz", k, q, level) for
    Helmholtz (one table of the tree's level)."""
    key: tuple
    dim: int
    kernel: str          # "laplace" | "helmholtz"
    k: float             # Helmholtz wave number (0 for Laplace)
    q: int
    level: int
    table_key: tuple
    n_points: int


def _nearest_level(dim, q, n):
    per = q ** dim
    levels = np.arange(1, 10)
    npts = (2 ** dim) ** levels * per
    return int(levels[np.argmin(np.abs(np.log(npts / n)))])


def config_c5(seed=5000, n_requests=10000, n_problems=800, n_range=(1e3, 5e5), qs=(3, 4, 5),
              k_range=(1, 30), densities_per_problem=4):
    """Serving mix: a catalogue of ``n_problems`` draws and ``n_requests``
    single-rhs requests over it.  A draw: dim 2 or 3 with equal
    probability, Laplace or Helmholtz with equal probability (k uniform in
    ``k_range``, a real number kept to 6 decimals, so every Helmholtz problem
    has its own table), N log-uniform in ``n_range`` realised as q uniform in
    ``qs`` and the uniform level whose N = 2^(dim L) q^dim is nearest to N in
    log (Laplace draws repeat problems: there are few (dim, q, level)).  A
    request picks a draw of the catalogue uniformly and one of its problem's
    ``densities_per_problem`` seeded Gaussian-sum densities (4..16 terms).

    Returns (problems {key: C5Problem}, requests [(key, density index)],
    density terms {key: [GaussianMixture]}).
    """
    rng = np.random.default_rng(seed)
    problems, catalogue = {}, []
    while len(catalogue) < n_problems:
        dim = 2 if rng.random() < 0.5 else 3
        kern = "laplace" if rng.random() < 0.5 else "helmholtz"
        k = round(float(rng.uniform(k_range[0], k_range[1])), 6) if kern == "helmholtz" else 0.0
        n = float(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        q = int(rng.choice(qs))
        lev = _nearest_level(dim, q, n)
        key = (dim, kern, k, q, lev)
        if key not in problems:
            # Laplace: one canonical table per (dim, q); Helmholtz: one table
            # of the tree's level for the problem's own k
            tkey = (dim, kern, 0.0, q) if kern == "laplace" else (dim, kern, k, q, lev)
            problems[key] = C5Problem(key, dim, kern, k, q, lev, tkey,
                                      (2 ** dim) ** lev * q ** dim)
        catalogue.append(key)   # a Laplace key drawn again counts again
    reqs = [(catalogue[int(rng.integers(n_problems))], int(rng.integers(densities_per_problem)))
            for _ in range(n_requests)]
    mixes = {}
    for key in sorted(problems):
        mixes[key] = [random_gaussian_mixture(rng, key[0], int(rng.integers(4, 17)),
                                              (0.01, 0.1))
                      for _ in range(densities_per_problem)]
    return problems, reqs, mixes


def c5_workloads(problems, seed=5000):
    """Trees and table sets of the serving problems: {key: Workload}.  Laplace
    uses one canonical table per (dim, q) with inferred scaling; Helmholtz one
    table of the tree's level for the problem's k (seeded values).  Problems
    of one tree shape share the tree (``meta["tree_key"]``) and problems of
    one tree and kernel share the schedule (``meta["sched_key"]``: every
    Helmholtz table set has one level, so the tile keys do not depend on k).
    """
    tables, trees = {}, {}
    out = {}
    for key in sorted(problems):
        p = problems[key]
        if p.table_key not in tables:
            tseed = seed + 7919 * p.dim + 101 * p.q + int(p.k * 1e6) + 13 * p.level
            if p.kernel == "laplace":
                tables[p.table_key] = synthetic_tables(p.dim, p.q, LaplaceKernel(p.dim),
                                                       seed=tseed, source_box_extent=1.0)
            else:
                tables[p.table_key] = synthetic_tables(
                    p.dim, p.q, HelmholtzKernel(p.dim), n_tables=1, seed=tseed,
                    source_box_extent=0.5 ** p.level, complex_values=True)
        tkey = (p.dim, p.q, p.level)
        if tkey not in trees:
            tree = build_uniform_tree(p.dim, p.level, p.q)
            trees[tkey] = build_list1_traversal(tree)
        trav = trees[tkey]
        kernel = LaplaceKernel(p.dim) if p.kernel == "laplace" else HelmholtzKernel(p.dim)
        out[key] = Workload(f"c5_{p.dim}d_{p.kernel}{p.k:g}_q{p.q}_l{p.level}", p.dim, p.q,
                            kernel, trav, tables[p.table_key], np.zeros((1, 0)), seed,
                            meta={"level": p.level, "table_key": p.table_key,
                                  "tree_key": tkey, "sched_key": (tkey, p.kernel)})
    return out


def config_c5_arrivals(seed=5500, n_new=12, n_range=(1e3, 2e5), qs=(3, 4, 5), k_range=(1, 30)):
    """Helmholtz problems that arrive while the serving mix runs: dim 2 or 3
    with equal probability, k uniform in ``k_range`` (a real number kept to 6
    decimals), N log-uniform in ``n_range`` realised as in :func:`config_c5`.
    Their tables do not exist yet: each is built on arrival by the FP64 GPU
    Duffy builder for its own k (:func:`c5_arrival_workloads`)."""
    rng = np.random.default_rng(seed)
    problems = {}
    while len(problems) < n_new:
        dim = 2 if rng.random() < 0.5 else 3
        k = round(float(rng.uniform(k_range[0], k_range[1])), 6)
        n = float(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        q = int(rng.choice(qs))
        lev = _nearest_level(dim, q, n)
        key = (dim, "helmholtz", k, q, lev)
        problems[key] = C5Problem(key, dim, "helmholtz", k, q, lev, (dim, "helmholtz", k, q, lev),
                                  (2 ** dim) ** lev * q ** dim)
    return problems


def c5_arrival_workloads(problems, seed=5500, build_ctas=0):
    """Trees of the arriving problems and, per problem, a function that
    builds its table set: one FP64 Duffy table (GPU, the reference's default
    orders) of the tree's level (source box extent 2^-level) for its k, on at
    most ``build_ctas`` CTAs when that is > 0.
    Returns ({key: Workload without tables}, {key: build function})."""
    import functools

    trees, out, builders = {}, {}, {}
    for key in sorted(problems):
        p = problems[key]
        tkey = (p.dim, p.q, p.level)
        if tkey not in trees:
            trees[tkey] = build_list1_traversal(build_uniform_tree(p.dim, p.level, p.q))
        kernel = HelmholtzKernel(p.dim)
        out[key] = Workload(f"c5_new_{p.dim}d_helmholtz{p.k:g}_q{p.q}_l{p.level}", p.dim, p.q,
                            kernel, trees[tkey], [], np.zeros((1, 0)), seed,
                            meta={"level": p.level, "table_key": p.table_key,
                                  "tree_key": tkey, "sched_key": (tkey, "helmholtz"),
                                  "tables": "duffy"})
        builders[key] = functools.partial(duffy_tables, p.dim, p.q, kernel, n_tables=1,
                                          source_box_extent=0.5 ** p.level, k=p.k,
                                          complex_values=True, max_ctas=build_ctas)
    return out, builders


def poisson_arrivals(n, rate, seed=0):
    """Arrival offsets (seconds) of a Poisson process of ``rate`` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def constant_workload(dim, q, level=1):
    """Completeness case: constant kernel table, density 1 on [-1, 1]^dim."""
    tree = build_uniform_tree(dim, level, q, a=-1.0, b=1.0)
    trav = build_list1_traversal(tree)
    t = NearFieldInteractionTable(q, dim=dim, sumpy_kernel=ConstantKernel(dim),
                                  source_box_extent=1.0)
    t.build_constant_table()
    return Workload(f"constant{dim}d_q{q}", dim, q, LaplaceKernel(dim), trav, [t],
                    np.ones((1, tree.ntargets)), 0)
