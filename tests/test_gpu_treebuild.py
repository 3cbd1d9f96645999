"""Box trees built on the GPU (``vl1_tree_balance``, ``vl1_tree_build_*``)
against the host builder (``tree_build``), array by array: the 2:1 level
restriction of a set of leaves (volumential/tree_interactive_build.py:202-432)
and the particle tree's layout (:1274-1441): box numbering, levels, integer
coordinates, centres, leaf flags, particle starts and counts, Gauss-Legendre
targets (bit for bit) and weights (to an ulp: the host raises the half
extent to the power dim with ``pow``)."""

import itertools

import numpy as np
import pytest

from volumential_gb300.tree_build import (
    _balance,
    build_adaptive_tree,
    build_adaptive_tree_device,
    build_list1_traversal,
    build_list1_traversal_device,
    build_tree_from_leaves,
    build_tree_from_leaves_device,
    build_uniform_tree,
)

pytestmark = pytest.mark.gpu


def _same_tree(h, d):
    assert (h.nboxes, h.aligned_nboxes) == (d.nboxes, d.aligned_nboxes)
    for name in ("box_levels", "box_coords", "box_centers", "box_is_leaf", "box_target_starts",
                 "box_target_counts_nonchild", "leaf_boxes", "targets", "level_start_box_nrs"):
        a, b = np.asarray(getattr(h, name)), np.asarray(getattr(d, name))
        assert a.shape == b.shape, name
        assert np.array_equal(a.astype(b.dtype) if a.dtype != b.dtype else a, b), name
    np.testing.assert_allclose(d.weights, h.weights, rtol=4e-16, atol=0)


def _leaves(tree):
    lv = tree.box_levels[tree.leaf_boxes]
    return lv, tree.box_coords[tree.leaf_boxes]


@pytest.mark.parametrize("dim,level,a,b", [(2, 5, -0.5, 0.5), (3, 3, -0.5, 0.5),
                                           (2, 4, -0.37, 0.91), (3, 2, -0.37, 0.91)])
def test_uniform_tree_equals_host(cuda, dim, level, a, b):
    h = build_uniform_tree(dim, level, 3, a=a, b=b)
    lv, co = _leaves(h)
    d = build_tree_from_leaves_device(lv, co, dim=dim, q_order=3, a=a, b=b, balance=False)
    _same_tree(h, d)


def _unbalanced_leaves(dim, rng, max_level):
    """Leaves of a random refinement, not 2:1 balanced."""
    kids = np.array(list(itertools.product((0, 1), repeat=dim)), dtype=np.int64)
    leaves = {}
    active = np.zeros((1, dim), dtype=np.int64)
    for lev in range(max_level + 1):
        split = rng.random(len(active)) < (0.9 if lev < 2 else 0.3)
        if lev == max_level:
            split[:] = False
        leaves[lev] = active[~split]
        active = (active[split][:, None, :] * 2 + kids[None]).reshape(-1, dim)
    return leaves


@pytest.mark.parametrize("dim,max_level,seed", [(2, 7, 1), (2, 9, 2), (3, 5, 3), (3, 6, 4)])
def test_balance_equals_host(cuda, dim, max_level, seed):
    rng = np.random.default_rng(seed)
    leaves = _unbalanced_leaves(dim, rng, max_level)
    lv = np.concatenate([np.full(len(c), l, np.uint8) for l, c in leaves.items()])
    co = np.concatenate([c for c in leaves.values()])
    host = build_tree_from_leaves(_balance({k: v.copy() for k, v in leaves.items()}, dim,
                                           max_level), dim=dim, q_order=2)
    dev = build_tree_from_leaves_device(lv, co, dim=dim, q_order=2, balance=True)
    _same_tree(host, dev)
    # and the list-1 CSR of the device tree is the host's
    hc, dc = build_list1_traversal(host), build_list1_traversal_device(dev)
    assert np.array_equal(hc.neighbor_source_boxes_lists, dc.neighbor_source_boxes_lists)


@pytest.mark.parametrize("dim,q,max_level", [(2, 3, 8), (3, 2, 6)])
def test_adaptive_refinement_equals_host(cuda, dim, q, max_level):
    """A criterion made of minima, maxima and separately rounded
    differences (no transcendental functions), evaluated with numpy on the
    host and with torch on the device: the same splits, the same tree.  A
    leaf splits when the point ``p`` lies within its nodes' bounding box
    widened by the box's own width on every side."""
    import torch

    p = [0.123, -0.271, 0.05][:dim]

    def near(nodes, lib):
        hit = None
        for ax in range(dim):
            if lib is np:
                lo, hi = nodes[ax].min(axis=-1), nodes[ax].max(axis=-1)
            else:
                lo, hi = nodes[ax].amin(dim=-1), nodes[ax].amax(dim=-1)
            w = hi - lo
            h = (lo - w <= p[ax]) & (p[ax] <= hi + w)
            hit = h if hit is None else hit & h
        return hit

    host = build_adaptive_tree(dim, q, lambda n: near(n, np), max_level=max_level, min_level=2)
    dev = build_adaptive_tree_device(dim, q, lambda n: near(n, torch), max_level=max_level,
                                     min_level=2)
    assert len(np.unique(host.box_levels[host.leaf_boxes])) >= 4
    _same_tree(host, dev)
