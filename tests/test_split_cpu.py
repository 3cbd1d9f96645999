"""Helmholtz split remainder: the product's series (restated from
``volumential/expansion_wrangler_fpnd.py:212-332, 4337-4378``) against the
closed form G_k - G_0 of the CPU restatement."""

import numpy as np
import pytest

from oracle import split_oracle as SO
from volumential_gb300.helmholtz_split import (
    remainder_coefficients,
    remainder_series,
    series_terms,
)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("k", [1.0, 7.5, 20.0, 12.0 + 0.5j])
def test_series_matches_the_closed_form(dim, k):
    r_max = 0.09
    n = series_terms(dim, k, r_max)
    r = np.concatenate([[0.0], np.geomspace(1e-7, r_max, 300)])
    got = remainder_series(dim, k, r, n)
    ref = SO.remainder(dim, k, r)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_series_term_counts():
    # the truncation rule of expansion_wrangler_fpnd.py:4337-4378
    assert series_terms(2, 0.0, 1.0) == 1 and series_terms(3, 0.0, 1.0) == 1
    assert series_terms(2, 20.0, 0.0663) == 12   # stops at n = 10 (+2)
    assert series_terms(3, 5.0, 0.0541) == 15    # stops at n = 13 (+2)
    assert series_terms(3, 1e6, 1.0) == 96
    c = remainder_coefficients(3, 2.0, 4)
    assert c.shape == (2, 5, 2)
    np.testing.assert_allclose(c[0, 1], [0.0, 2.0 / (4 * np.pi)], rtol=1e-15)


def test_max_neighbor_distance_follows_the_coarsest_active_box():
    from volumential_gb300.helmholtz_split import max_neighbor_distance
    from volumential_gb300.tree_build import build_uniform_tree

    t = build_uniform_tree(2, 3, 2)
    assert t.dimensions == 2
    assert abs(max_neighbor_distance(t) - 2 * np.sqrt(2) * t.root_extent / 8) < 1e-15
