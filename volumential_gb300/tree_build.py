"""Box trees with tensor Gauss-Legendre nodes on the leaves, and their list-1
(neighbour source box) CSR.

Host-side builder for the inputs of the list-1 evaluation.  It follows the
layout of ``volumential/tree_interactive_build.py:1274-1441``
(``build_particle_tree_from_box_tree``) and of boxtree's traversal:

* boxes are numbered level by level (root = box 0), ``box_levels`` is uint8,
  ``box_centers`` is ``[dim, aligned_nboxes]`` with ``aligned_nboxes`` rounded
  up to a multiple of 32 (``tree_interactive_build.py:1356``);
* particles are the ``q**dim`` Gauss-Legendre nodes of every leaf, stored
  box-contiguously; inside a leaf they follow ``meshgrid(indexing="ij")``
  order, so the box-local index is the mode id with axis 0 slowest
  (``meshgen.py:979-998``) and ``sorted_target_ids`` is the identity;
* sources are targets (``sources_are_targets=True``);
* list 1 of a leaf is every leaf whose closure touches it, itself included.

Adaptive trees are refined by a user criterion and then 2:1 balanced over
faces, edges and corners (``tree_interactive_build.py:202-432``), so every
list-1 pair is a case of the list-1 gallery.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "ParticleTree",
    "Traversal",
    "gauss_legendre_unit",
    "build_uniform_tree",
    "build_adaptive_tree",
    "build_tree_from_leaves",
    "build_list1_traversal",
    "build_list1_traversal_device",
    "build_tree_from_leaves_device",
    "build_adaptive_tree_device",
]


def gauss_legendre_unit(q_order):
    """Nodes (ascending) and weights of the q-point Gauss-Legendre rule on [-1, 1]."""
    x, w = np.polynomial.legendre.leggauss(int(q_order))
    return x, w


@dataclass
class ParticleTree:
    dim: int
    q_order: int
    root_extent: float
    root_vertex: np.ndarray
    nboxes: int
    aligned_nboxes: int
    box_centers: np.ndarray          # f64 [dim, aligned_nboxes]
    box_levels: np.ndarray           # u8 [nboxes]
    box_coords: np.ndarray           # i64 [nboxes, dim] integer box index on its level
    box_is_leaf: np.ndarray          # bool [nboxes]
    box_target_starts: np.ndarray    # i32 [nboxes]
    box_target_counts_nonchild: np.ndarray  # i32 [nboxes]
    leaf_boxes: np.ndarray           # i32 [nleaves], in particle order
    targets: np.ndarray              # f64 [dim, N]
    weights: np.ndarray              # f64 [N] quadrature weights
    level_start_box_nrs: np.ndarray  # i32 [nlevels + 1]
    sources_are_targets: bool = True

    @property
    def ntargets(self):
        return int(self.targets.shape[1])

    @property
    def nsources(self):
        return self.ntargets

    @property
    def sources(self):
        return self.targets

    @property
    def dimensions(self):
        """boxtree's name of the dimension."""
        return self.dim

    @property
    def box_source_starts(self):
        return self.box_target_starts

    @property
    def box_source_counts_nonchild(self):
        return self.box_target_counts_nonchild

    @property
    def sorted_target_ids(self):
        return np.arange(self.ntargets, dtype=np.int32)

    @property
    def user_source_ids(self):
        return np.arange(self.ntargets, dtype=np.int32)

    @property
    def nlevels(self):
        return int(self.box_levels.max()) + 1 if self.nboxes else 0

    def box_local_mode_ids(self):
        """Box-local particle index (``expansion_wrangler_fpnd.py:408-424``)."""
        nq = self.q_order ** self.dim
        return np.tile(np.arange(nq, dtype=np.int32), self.ntargets // nq)


@dataclass
class Traversal:
    tree: ParticleTree
    target_boxes: np.ndarray                   # i32 [n_tgt_boxes]
    neighbor_source_boxes_starts: np.ndarray   # i32 [n_tgt_boxes + 1]
    neighbor_source_boxes_lists: np.ndarray    # i32 [nnz]
    extra: dict = field(default_factory=dict)

    @property
    def nnz(self):
        lists = self.neighbor_source_boxes_lists
        return int(lists.numel() if hasattr(lists, "numel") else lists.size)


# {{{ keys: one int64 per (level, integer coordinates)

def _level_offsets(dim, max_level):
    sizes = [1 << (dim * lev) for lev in range(max_level + 2)]
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)


def _lin(coords, level):
    coords = np.asarray(coords, dtype=np.int64)
    out = np.zeros(coords.shape[:-1], dtype=np.int64)
    for a in range(coords.shape[-1]):
        out = (out << np.int64(level)) | coords[..., a]
    return out

# }}}


def _balance(leaves_by_level, dim, max_level):
    """Refine leaves until adjacent leaves differ by at most one level."""
    deltas = np.array(list(itertools.product((-1, 0, 1), repeat=dim)), dtype=np.int64)
    while True:
        offs = _level_offsets(dim, max_level)
        keys = np.sort(np.concatenate(
            [offs[lev] + _lin(c, lev) for lev, c in leaves_by_level.items() if len(c)]))
        to_refine = {}
        # A leaf at level L forces every leaf that contains a same-level
        # neighbour position and sits at level < L-1 to split.
        for lev in sorted(leaves_by_level, reverse=True):
            c = leaves_by_level[lev]
            if len(c) == 0 or lev < 2:
                continue
            npos = (c[:, None, :] + deltas[None, :, :]).reshape(-1, dim)
            inside = np.all((npos >= 0) & (npos < (1 << lev)), axis=1)
            npos = npos[inside]
            for coarse in range(0, lev - 1):
                cc = npos >> (lev - coarse)
                k = offs[coarse] + _lin(cc, coarse)
                pos = np.searchsorted(keys, k)
                pos = np.minimum(pos, len(keys) - 1)
                hit = keys[pos] == k
                if np.any(hit):
                    to_refine.setdefault(coarse, []).append(np.unique(cc[hit], axis=0))
        if not to_refine:
            return leaves_by_level
        for lev, lst in to_refine.items():
            split = np.unique(np.concatenate(lst), axis=0)
            cur = leaves_by_level[lev]
            cur_k = _lin(cur, lev)
            keep = ~np.isin(cur_k, _lin(split, lev))
            leaves_by_level[lev] = cur[keep]
            kids = (split[:, None, :] * 2 + np.array(
                list(itertools.product((0, 1), repeat=dim)), dtype=np.int64)[None]
                    ).reshape(-1, dim)
            nxt = leaves_by_level.get(lev + 1, np.zeros((0, dim), dtype=np.int64))
            leaves_by_level[lev + 1] = np.concatenate([nxt, kids])
            max_level = max(max_level, lev + 1)


def build_tree_from_leaves(leaves_by_level, *, dim, q_order, a=-0.5, b=0.5):
    """Assemble a :class:`ParticleTree` from leaf integer coordinates per level."""
    dim = int(dim)
    q = int(q_order)
    root_extent = float(b - a)
    root_vertex = np.full(dim, float(a))
    levels = sorted(lev for lev, c in leaves_by_level.items() if len(c))
    max_level = levels[-1]

    # all boxes: leaves plus their ancestors
    per_level = {lev: np.zeros((0, dim), dtype=np.int64) for lev in range(max_level + 1)}
    leaf_keys = set()
    for lev in levels:
        c = np.asarray(leaves_by_level[lev], dtype=np.int64)
        per_level[lev] = np.concatenate([per_level[lev], c])
        leaf_keys.update((lev, int(k)) for k in _lin(c, lev).tolist())
        anc = c
        for up in range(lev - 1, -1, -1):
            anc = np.unique(anc >> 1, axis=0)
            per_level[up] = np.concatenate([per_level[up], anc])
    coords_list, lev_list = [], []
    for lev in range(max_level + 1):
        c = np.unique(per_level[lev], axis=0)   # lexicographic order
        coords_list.append(c)
        lev_list.append(np.full(len(c), lev, dtype=np.uint8))
    box_coords = np.concatenate(coords_list)
    box_levels = np.concatenate(lev_list)
    nboxes = len(box_levels)
    aligned = ((nboxes + 31) // 32) * 32
    level_start = np.concatenate([[0], np.cumsum([len(c) for c in coords_list])]).astype(np.int32)

    extents = root_extent / (2.0 ** box_levels.astype(np.float64))
    centers = np.zeros((dim, aligned), dtype=np.float64)
    centers[:, :nboxes] = (root_vertex[:, None]
                           + (box_coords.T.astype(np.float64) + 0.5) * extents[None, :])

    is_leaf = np.array([(int(l), int(k)) in leaf_keys for l, k in zip(
        box_levels.tolist(),
        np.concatenate([_lin(c, lev) for lev, c in enumerate(coords_list)]).tolist())])

    leaf_boxes = np.flatnonzero(is_leaf).astype(np.int32)
    nq = q ** dim
    starts = np.zeros(nboxes, dtype=np.int32)
    counts = np.zeros(nboxes, dtype=np.int32)
    starts[leaf_boxes] = np.arange(len(leaf_boxes), dtype=np.int32) * nq
    counts[leaf_boxes] = nq
    # non-leaf boxes point at their first descendant's particles (unused)

    x, w = gauss_legendre_unit(q)
    grids = np.meshgrid(*([x] * dim), indexing="ij")
    ref = np.stack([g.ravel() for g in grids], axis=0)       # [dim, nq]
    wgrid = np.meshgrid(*([w] * dim), indexing="ij")
    wref = np.prod(np.stack([g.ravel() for g in wgrid], axis=0), axis=0)
    lc = centers[:, leaf_boxes]                               # [dim, nleaves]
    le = extents[leaf_boxes]
    targets = (lc[:, :, None] + 0.5 * le[None, :, None] * ref[:, None, :]).reshape(dim, -1)
    weights = ((0.5 * le[:, None]) ** dim * wref[None, :]).reshape(-1)

    return ParticleTree(
        dim=dim, q_order=q, root_extent=root_extent, root_vertex=root_vertex,
        nboxes=nboxes, aligned_nboxes=aligned, box_centers=centers,
        box_levels=box_levels, box_coords=box_coords, box_is_leaf=is_leaf,
        box_target_starts=starts, box_target_counts_nonchild=counts,
        leaf_boxes=leaf_boxes, targets=np.ascontiguousarray(targets),
        weights=np.ascontiguousarray(weights), level_start_box_nrs=level_start)


def build_uniform_tree(dim, level, q_order, a=-0.5, b=0.5):
    """Complete tree whose leaves are all at ``level`` on ``[a, b]^dim``."""
    n = 1 << int(level)
    c = np.array(list(itertools.product(range(n), repeat=dim)), dtype=np.int64)
    return build_tree_from_leaves({int(level): c}, dim=dim, q_order=q_order, a=a, b=b)


def build_adaptive_tree(dim, q_order, refine_fn, *, max_level, min_level=0,
                        a=-0.5, b=0.5, max_leaves=None):
    """2:1-balanced adaptive tree.

    ``refine_fn(nodes[dim, nboxes, nq]) -> bool[nboxes]`` decides, from the
    values of the leaf's Gauss-Legendre nodes, whether a leaf splits.  Leaves
    below ``min_level`` always split; none splits beyond ``max_level``.
    """
    dim = int(dim)
    root_extent = float(b - a)
    x, _ = gauss_legendre_unit(q_order)
    grids = np.meshgrid(*([x] * dim), indexing="ij")
    ref = np.stack([g.ravel() for g in grids], axis=0)
    kids = np.array(list(itertools.product((0, 1), repeat=dim)), dtype=np.int64)

    leaves = {}
    active = np.zeros((1, dim), dtype=np.int64)
    for lev in range(0, int(max_level) + 1):
        if len(active) == 0:
            break
        if lev < min_level:
            split = np.ones(len(active), dtype=bool)
        elif lev == max_level:
            split = np.zeros(len(active), dtype=bool)
        else:
            ext = root_extent / 2 ** lev
            ctr = a + (active.astype(np.float64) + 0.5) * ext          # [n, dim]
            nodes = ctr.T[:, :, None] + 0.5 * ext * ref[:, None, :]    # [dim, n, nq]
            split = np.asarray(refine_fn(nodes), dtype=bool)
        leaves[lev] = active[~split]
        active = (active[split][:, None, :] * 2 + kids[None]).reshape(-1, dim)
        if max_leaves is not None and sum(len(v) for v in leaves.values()) + len(active) > max_leaves:
            raise ValueError("adaptive tree exceeds max_leaves")
    leaves = _balance({k: v for k, v in leaves.items()}, dim, int(max_level))
    return build_tree_from_leaves(leaves, dim=dim, q_order=q_order, a=a, b=b)


def build_list1_traversal(tree: ParticleTree) -> Traversal:
    """Target boxes (leaves) and their list-1 source boxes as CSR."""
    dim = tree.dim
    levels = tree.box_levels.astype(np.int64)
    max_level = int(levels.max())
    offs = _level_offsets(dim, max_level)
    keys = offs[levels] + _lin_per_box(tree.box_coords, levels)
    is_leaf = tree.box_is_leaf
    leaf_key_sorted_idx = np.argsort(keys[is_leaf])
    leaf_keys = keys[is_leaf][leaf_key_sorted_idx]
    leaf_ids = np.flatnonzero(is_leaf)[leaf_key_sorted_idx]

    def lookup(k):
        pos = np.minimum(np.searchsorted(leaf_keys, k), len(leaf_keys) - 1)
        hit = leaf_keys[pos] == k
        return np.where(hit, leaf_ids[pos], -1)

    deltas = np.array(list(itertools.product((-1, 0, 1), repeat=dim)), dtype=np.int64)
    fine = np.array(list(itertools.product((-1, 0, 1, 2), repeat=dim)), dtype=np.int64)
    fine = fine[~np.all((fine >= 0) & (fine <= 1), axis=1)]

    targets = tree.leaf_boxes.astype(np.int64)
    tl = levels[targets]
    tc = tree.box_coords[targets]
    cand = []
    # same level and one level coarser
    for lev_shift in (0, 1):
        for d in deltas:
            pos = tc + d
            clev = tl - lev_shift
            valid = np.all((pos >= 0) & (pos < (1 << tl)[:, None]), axis=1) & (clev >= 0)
            cpos = pos >> lev_shift
            k = np.where(valid, offs[np.maximum(clev, 0)] + _lin_per_box(cpos, np.maximum(clev, 0)), -1)
            ids = np.where(valid, lookup(k), -1)
            if lev_shift == 1:
                # a coarser box containing the leaf itself is its ancestor, never a leaf
                ids = np.where(np.all(cpos == (tc >> 1), axis=1), -1, ids)
            cand.append(ids)
    # one level finer
    for d in fine:
        pos = 2 * tc + d
        flev = tl + 1
        valid = np.all((pos >= 0) & (pos < (1 << flev)[:, None]), axis=1) & (flev <= max_level)
        k = np.where(valid, offs[np.minimum(flev, max_level)] +
                     _lin_per_box(np.where(valid[:, None], pos, 0), np.minimum(flev, max_level)), -1)
        cand.append(np.where(valid, lookup(k), -1))
    cand = np.sort(np.stack(cand, axis=1), axis=1)
    keep = cand >= 0
    keep[:, 1:] &= cand[:, 1:] != cand[:, :-1]
    nnz_per = keep.sum(axis=1)
    starts = np.concatenate([[0], np.cumsum(nnz_per)]).astype(np.int32)
    flat = cand[keep].astype(np.int32)
    return Traversal(tree=tree, target_boxes=tree.leaf_boxes.astype(np.int32),
                     neighbor_source_boxes_starts=starts,
                     neighbor_source_boxes_lists=flat)


def _lin_per_box(coords, levels):
    """Linear index of integer coordinates with a per-row level."""
    coords = np.asarray(coords, dtype=np.int64)
    levels = np.asarray(levels, dtype=np.int64)
    out = np.zeros(coords.shape[0], dtype=np.int64)
    for a in range(coords.shape[1]):
        out = (out << levels) | coords[:, a]
    return out


def build_list1_traversal_device(tree: ParticleTree, stream=None, as_numpy=True) -> Traversal:
    """The list-1 CSR of ``tree`` computed on the GPU (``vl1_list1_csr``);
    the same arrays as :func:`build_list1_traversal`.  ``as_numpy=False``
    keeps the CSR as CUDA tensors."""
    import ctypes as C

    import torch

    from . import _lib

    dim = tree.dim

    def dev(a, dt):   # host arrays or CUDA tensors of a tree built on the device
        if torch.is_tensor(a):
            return a.to(device="cuda", dtype=dt).contiguous()
        return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dt)

    levels = dev(tree.box_levels, torch.uint8)
    coords = dev(tree.box_coords, torch.int32)
    lv = dev(tree.leaf_boxes, torch.int32)
    n_leaves = int(lv.numel())
    leaves = lv.cpu().numpy() if as_numpy else lv
    lib = _lib.lib()
    ws = torch.empty(int(lib.vl1_list1_csr_workspace_bytes(n_leaves)), dtype=torch.uint8,
                     device="cuda")
    cap = n_leaves * (110 if dim == 3 else 30)
    starts = torch.empty(n_leaves + 1, dtype=torch.int32, device="cuda")
    lists = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    d = _lib.CsrDesc()
    d.dim, d.nboxes, d.n_leaves = dim, int(tree.nboxes), n_leaves
    d.max_level = int(levels.max()) if n_leaves else 0
    d.box_levels, d.box_coords, d.leaf_boxes = levels.data_ptr(), coords.data_ptr(), lv.data_ptr()
    d.starts, d.lists, d.lists_capacity = starts.data_ptr(), lists.data_ptr(), cap
    d.workspace, d.workspace_bytes = ws.data_ptr(), ws.numel()
    nnz = C.c_int64()
    sh = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _lib.check(lib.vl1_list1_csr(C.byref(d), C.byref(nnz), C.c_void_p(sh)), "vl1_list1_csr")
    lists = lists[: nnz.value]
    if as_numpy:
        return Traversal(tree=tree, target_boxes=leaves,
                         neighbor_source_boxes_starts=starts.cpu().numpy(),
                         neighbor_source_boxes_lists=lists.cpu().numpy())
    return Traversal(tree=tree, target_boxes=lv, neighbor_source_boxes_starts=starts,
                     neighbor_source_boxes_lists=lists)



# {{{ trees built on the device

def _ref_rule(dim, q):
    """Reference nodes [dim, q^dim] on [-1, 1] (meshgrid "ij") and the
    products of their weights [q^dim], as the host builder forms them."""
    x, w = gauss_legendre_unit(q)
    grids = np.meshgrid(*([x] * dim), indexing="ij")
    ref = np.stack([g.ravel() for g in grids], axis=0)
    wgrid = np.meshgrid(*([w] * dim), indexing="ij")
    wref = np.prod(np.stack([g.ravel() for g in wgrid], axis=0), axis=0)
    return np.ascontiguousarray(ref), np.ascontiguousarray(wref)


def build_tree_from_leaves_device(leaf_levels, leaf_coords, *, dim, q_order, a=-0.5, b=0.5,
                                  balance=True, stream=None, as_numpy=True):
    """:func:`build_tree_from_leaves` on the GPU (``vl1_tree_balance``,
    ``vl1_tree_build_*``): optional 2:1 level restriction of the leaves
    (``leaf_levels`` [n] and integer ``leaf_coords`` [n, dim], device or host
    arrays), then the boxes, centres and Gauss-Legendre particles.  The
    arrays equal the host builder's (the weights to an ulp: the host raises
    the half extent to the power dim with ``pow``).  ``as_numpy=False``
    returns a tree whose arrays are CUDA tensors."""
    import ctypes as C

    import torch

    from . import _lib

    dim, q = int(dim), int(q_order)
    lib = _lib.lib()
    sh = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    lv = torch.as_tensor(np.asarray(leaf_levels) if not torch.is_tensor(leaf_levels)
                         else leaf_levels).to(device="cuda", dtype=torch.uint8)
    co = torch.as_tensor(np.asarray(leaf_coords) if not torch.is_tensor(leaf_coords)
                         else leaf_coords).to(device="cuda", dtype=torch.int32).reshape(-1, dim)
    n = int(lv.numel())
    if balance:
        cap = max(n, 1) * 4 + 64
        while True:
            lvb = torch.empty(cap, dtype=torch.uint8, device="cuda")
            cob = torch.empty((cap, dim), dtype=torch.int32, device="cuda")
            lvb[:n] = lv
            cob[:n] = co
            nn = C.c_int32(n)
            st = lib.vl1_tree_balance(dim, C.byref(nn), cap, lvb.data_ptr(), cob.data_ptr(),
                                      C.c_void_p(sh))
            if st == _lib.VL1_E_ARG and "capacity" in _lib.last_error():
                cap *= 4
                continue
            _lib.check(st, "vl1_tree_balance")
            lv, co, n = lvb[:nn.value], cob[:nn.value].contiguous(), nn.value
            break
    root_extent = float(b - a)
    rv = np.full(dim, float(a))
    sizes = (C.c_int32 * 3)()
    bld = C.c_void_p()
    _lib.check(lib.vl1_tree_build_begin(dim, q, n, lv.data_ptr(), co.data_ptr(), root_extent,
                                        rv.ctypes.data, C.byref(bld), sizes, C.c_void_p(sh)),
               "vl1_tree_build_begin")
    try:
        nboxes, aligned, max_level = int(sizes[0]), int(sizes[1]), int(sizes[2])
        level_start = np.empty(max_level + 2, dtype=np.int32)
        _lib.check(lib.vl1_tree_build_level_starts(bld, level_start.ctypes.data),
                   "vl1_tree_build_level_starts")
        nq = q ** dim
        ref, wref = _ref_rule(dim, q)
        dev = lambda shape, dt: torch.empty(shape, dtype=dt, device="cuda")  # noqa: E731
        out = {"levels": dev(nboxes, torch.uint8), "coords": dev((nboxes, dim), torch.int32),
               "centers": dev((dim, aligned), torch.float64),
               "is_leaf": dev(nboxes, torch.uint8), "starts": dev(nboxes, torch.int32),
               "counts": dev(nboxes, torch.int32), "leaf_boxes": dev(n, torch.int32),
               "targets": dev((dim, n * nq), torch.float64),
               "weights": dev(n * nq, torch.float64)}
        _lib.check(lib.vl1_tree_build_fill(
            bld, ref.ctypes.data, wref.ctypes.data, out["levels"].data_ptr(),
            out["coords"].data_ptr(), out["centers"].data_ptr(), out["is_leaf"].data_ptr(),
            out["starts"].data_ptr(), out["counts"].data_ptr(), out["leaf_boxes"].data_ptr(),
            out["targets"].data_ptr(), out["weights"].data_ptr(), C.c_void_p(sh)),
            "vl1_tree_build_fill")
    finally:
        lib.vl1_tree_builder_destroy(bld)
    cv = (lambda t: t.cpu().numpy()) if as_numpy else (lambda t: t)
    return ParticleTree(
        dim=dim, q_order=q, root_extent=root_extent, root_vertex=rv, nboxes=nboxes,
        aligned_nboxes=aligned, box_centers=cv(out["centers"]), box_levels=cv(out["levels"]),
        box_coords=cv(out["coords"].to(torch.int64)),
        box_is_leaf=cv(out["is_leaf"].to(torch.bool)), box_target_starts=cv(out["starts"]),
        box_target_counts_nonchild=cv(out["counts"]), leaf_boxes=cv(out["leaf_boxes"]),
        targets=cv(out["targets"]), weights=cv(out["weights"]), level_start_box_nrs=level_start)


def build_adaptive_tree_device(dim, q_order, refine_fn, *, max_level, min_level=0, a=-0.5,
                               b=0.5, stream=None, as_numpy=True):
    """:func:`build_adaptive_tree` with the tree on the GPU: per level, the
    nodes of the active boxes are formed on the device and
    ``refine_fn(nodes)`` (a CUDA tensor [dim, n_boxes, q^dim] -> bool tensor
    [n_boxes], e.g. a density's variation over a leaf) decides the splits;
    then the 2:1 restriction and the assembly run on the device."""
    import itertools as it

    import torch

    dim, q = int(dim), int(q_order)
    root_extent = float(b - a)
    ref = torch.from_numpy(_ref_rule(dim, q)[0]).to("cuda")
    kids = torch.tensor(list(it.product((0, 1), repeat=dim)), dtype=torch.int64, device="cuda")
    lev_list, coord_list = [], []
    active = torch.zeros((1, dim), dtype=torch.int64, device="cuda")
    for lev in range(0, int(max_level) + 1):
        if active.shape[0] == 0:
            break
        if lev < min_level:
            split = torch.ones(active.shape[0], dtype=torch.bool, device="cuda")
        elif lev == max_level:
            split = torch.zeros(active.shape[0], dtype=torch.bool, device="cuda")
        else:
            ext = root_extent / 2 ** lev
            ctr = a + (active.to(torch.float64) + 0.5) * ext
            nodes = ctr.T[:, :, None] + 0.5 * ext * ref[:, None, :]
            split = torch.as_tensor(refine_fn(nodes), device="cuda").to(torch.bool)
        keep = active[~split]
        lev_list.append(torch.full((keep.shape[0],), lev, dtype=torch.uint8, device="cuda"))
        coord_list.append(keep)
        active = (active[split][:, None, :] * 2 + kids[None]).reshape(-1, dim)
    levels = torch.cat(lev_list)
    coords = torch.cat(coord_list).to(torch.int32)
    return build_tree_from_leaves_device(levels, coords, dim=dim, q_order=q, a=a, b=b,
                                         balance=True, stream=stream, as_numpy=as_numpy)

# }}}
