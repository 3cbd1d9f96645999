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


@pytest.mark.parametrize("dim,k", [(2, 20.0), (3, 7.0), (2, 12.0 + 0.5j), (3, 5.0 + 0.3j)])
@pytest.mark.parametrize("order", [2, 3])
def test_split_orders_move_terms_out_of_the_series(dim, k, order):
    # expansion_wrangler_fpnd.py:212-332 (terms left in the remainder) and
    # :5052-5115 (the extracted terms' coefficients)
    from volumential_gb300.helmholtz_split import split_extra_terms

    r_max = 0.09
    n = series_terms(dim, k, r_max)
    r = np.concatenate([[0.0], np.geomspace(1e-7, r_max, 300)])
    got = remainder_series(dim, k, r, n, order)
    ref = SO.remainder(dim, k, r, order)
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    terms = split_extra_terms(dim, k, order)
    want = SO.extracted_terms(dim, k, order)
    assert [key for key, _ in terms] == [(kind, p) for kind, p, _ in want]
    for (_, c), (_, _, cw) in zip(terms, want):
        assert abs(c - cw) <= 1e-14 * abs(cw)
    # the series with the extracted terms added back is the order-1 series
    back = got + sum(c * SO.radial_term(kind, p, r) for kind, p, c in want)
    assert np.max(np.abs(back - remainder_series(dim, k, r, n, 1))) <= 1e-13 * np.max(
        np.abs(ref))


def test_split_term_keys_scaling_codes_and_key_forms():
    from volumential_gb300.expansion_wrangler_fpnd import _normalize_term_key
    from volumential_gb300.helmholtz_split import split_term_keys, term_scaling_code
    from volumential_gb300.list1 import parse_scaling_code

    assert split_term_keys(2, 1) == [] and split_term_keys(3, 1) == []
    assert split_term_keys(2, 3) == [("power_log", 2), ("power_log", 4)]
    assert split_term_keys(3, 3) == [("power", 1), ("power", 3)]
    # (h / h0)^(dim + power): expansion_wrangler_fpnd.py:4777-4799
    for dim, p in [(2, 2), (2, 4), (3, 1), (3, 3)]:
        code = term_scaling_code(dim, p).replace("BOX", "sbox")
        assert parse_scaling_code(code) == dim + p
    assert _normalize_term_key(("power_log", 2)) == ("power_log", 2)
    assert _normalize_term_key(3) == ("power", 3)
    assert _normalize_term_key("constant") == ("power", 0)
    assert _normalize_term_key("power:5") == ("power", 5)
    assert _normalize_term_key("power_log:4") == ("power_log", 4)
    for bad in [("power_log", 0), ("power", -1), ("cube", 2), "power-log:2", 2.5]:
        with pytest.raises((ValueError, TypeError)):
            _normalize_term_key(bad)


def test_log_alpha_per_source_follows_the_boxes():
    # expansion_wrangler_fpnd.py:4909-4974 on an adaptive tree
    from volumential_gb300.helmholtz_split import log_alpha_per_source
    from volumential_gb300.tree_build import build_adaptive_tree

    def refine(nodes):   # boxes with a node near (0.3, 0.3)
        return (np.linalg.norm(nodes - 0.3, axis=0) < 0.2).any(axis=1)

    tree = build_adaptive_tree(2, 3, refine, max_level=4, min_level=1)
    got = log_alpha_per_source(tree, 0.25)
    ref = SO.log_alpha(tree.box_levels, tree.box_source_starts,
                       tree.box_source_counts_nonchild, tree.root_extent, 0.25)
    assert np.array_equal(got, ref)
    assert len(np.unique(got)) > 1


def test_automatic_split_order_planner():
    # expansion_wrangler_fpnd.py:385-405, 4252-4323
    from volumential_gb300.helmholtz_split import (
        choose_auto_split_order,
        select_split_order_from_rho,
    )

    assert select_split_order_from_rho(0.1, (0.5, 1.5, 3.0), (2, 3, 4, 5)) == 2
    assert select_split_order_from_rho(1.5, (0.5, 1.5, 3.0), (2, 3, 4, 5)) == 3
    assert select_split_order_from_rho(9.0, (0.5, 1.5, 3.0), (2, 3, 4, 5)) == 5
    with pytest.raises(ValueError):
        select_split_order_from_rho(1.0, (0.5,), (2, 3, 4))
    # geometric ladders: real 0.25 * 2^j, imaginary 0.5 * 2^j over orders 2..12
    order, info = choose_auto_split_order({}, 0.3, 0.0)
    assert order == 3 and info["orders"] == tuple(range(2, 13))
    order, _ = choose_auto_split_order({}, 0.3, 1.9)
    assert order == 4   # the imaginary part asks for more
    order, info = choose_auto_split_order({}, 1e3, 0.0)
    assert order == 12 and info["beyond_coverage"]
    order, _ = choose_auto_split_order({"rho_thresholds": (0.5, 1.5, 3.0)}, 1.0, 0.0)
    assert order == 3
    order, _ = choose_auto_split_order({"orders": (1, 2), "rho_thresholds": (0.7,)}, 0.5, 0.0)
    assert order == 1


def test_wrangler_chooses_the_split_order_from_rho():
    from volumential_gb300 import workloads as W
    from volumential_gb300.expansion_wrangler_fpnd import (
        FPNDExpansionWrangler,
        FPNDTreeIndependentDataForWrangler,
    )
    from volumential_gb300.helmholtz_split import split_rho_components
    from volumential_gb300.kernels import HelmholtzKernel, LaplaceKernel
    from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

    w = W.uniform_workload("auto", 2, 3, 3, kernel=HelmholtzKernel(2))
    lap = NearFieldInteractionTable(3, dim=2, sumpy_kernel=LaplaceKernel(2),
                                    source_box_extent=w.tree.root_extent)
    ti = FPNDTreeIndependentDataForWrangler(target_kernels=[HelmholtzKernel(2)])
    wr = FPNDExpansionWrangler(ti, w.traversal, [lap], dtype=np.complex128, quad_order=3,
                               kernel_extra_kwargs={"k": 20.0}, helmholtz_split_order="auto")
    rho_r, rho_i = split_rho_components(w.tree, [20.0])
    assert rho_r == 20.0 * w.tree.root_extent / 8 and rho_i == 0.0
    assert wr.helmholtz_split_order == wr.helmholtz_split_auto_selection["order"]
    # rho 2.5: thresholds 0.25, 0.5, 1, 2, 4, ...: the fifth (4) is the first
    # not exceeded, order 2 + 4
    assert wr.helmholtz_split_order == 6
    # several output kernels: clamped to order 1, as the reference does
    ti2 = FPNDTreeIndependentDataForWrangler(
        target_kernels=[HelmholtzKernel(2), HelmholtzKernel(2, helmholtz_k_name="k2")])
    wr2 = FPNDExpansionWrangler(ti2, w.traversal, [lap], dtype=np.complex128, quad_order=3,
                                kernel_extra_kwargs={"k": 20.0, "k2": 5.0},
                                helmholtz_split_order=3)
    assert wr2.helmholtz_split_order == 1
    with pytest.raises(ValueError):
        FPNDExpansionWrangler(ti, w.traversal, [lap], dtype=np.complex128, quad_order=3,
                              kernel_extra_kwargs={"k": 20.0},
                              helmholtz_split_auto_config={
                                  "power_log_single_table_beta_mode": "other"})
