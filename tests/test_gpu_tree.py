"""List-1 CSR built on the GPU (``vl1_list1_csr``) against the host builder
(``tree_build.build_list1_traversal``), bit for bit, on uniform and adaptive
2:1-balanced trees."""

import numpy as np
import pytest

from volumential_gb300 import workloads as W
from volumential_gb300.tree_build import (
    build_adaptive_tree,
    build_list1_traversal,
    build_list1_traversal_device,
    build_uniform_tree,
)

pytestmark = pytest.mark.gpu


def _same(tree):
    h = build_list1_traversal(tree)
    d = build_list1_traversal_device(tree)
    np.testing.assert_array_equal(h.target_boxes, d.target_boxes)
    np.testing.assert_array_equal(h.neighbor_source_boxes_starts,
                                  d.neighbor_source_boxes_starts)
    np.testing.assert_array_equal(h.neighbor_source_boxes_lists,
                                  d.neighbor_source_boxes_lists)
    return h


@pytest.mark.parametrize("dim,level", [(2, 1), (2, 3), (2, 6), (3, 1), (3, 2), (3, 4)])
def test_uniform_trees(cuda, dim, level):
    h = _same(build_uniform_tree(dim, level, 2))
    n = 1 << level
    assert h.nnz == ((3 * n - 2) ** dim if n > 1 else 1)


@pytest.mark.parametrize("dim,tol,max_level", [(2, 3e-2, 7), (3, 3e-2, 5)])
def test_adaptive_trees(cuda, dim, tol, max_level):
    mix = W.random_gaussian_mixture(np.random.default_rng(dim), dim, 12, (0.01, 0.08))

    def refine(nodes):
        v = mix(nodes)
        return (v.max(axis=-1) - v.min(axis=-1)) > tol

    tree = build_adaptive_tree(dim, 3, refine, max_level=max_level, min_level=2)
    assert len(np.unique(tree.box_levels[tree.box_is_leaf])) >= 3
    _same(tree)


def test_c2_tree(cuda):
    w = W.config_c2(tables="synthetic")
    _same(w.tree)
