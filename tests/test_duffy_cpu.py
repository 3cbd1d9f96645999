"""Duffy radial table builder, host side: 1D rules and entry geometry of the
product against rules generated by the reference
(``tests/golden/duffy_golden.npz``, ``make_duffy_golden.py``), and the CPU
restatement (``oracle/duffy_oracle.py``) pinned to the reference's own scalar
Duffy integrator on the same entries, plus the reference's known answers
(``test/test_duffy_batched_manufactured.py:129-284``)."""

import os

import numpy as np
import pytest

from oracle import duffy_oracle as DO
from volumential_gb300 import table_builder as TB
from volumential_gb300.kernels import LaplaceKernel
from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "duffy_golden.npz"))
KIND = {0: "laplace", 1: "helmholtz"}


@pytest.mark.parametrize("n", [11, 21, 31, 61])
def test_radial_rules_match_the_reference(n):
    x, w = TB.tanh_sinh_fast_rule(n)
    np.testing.assert_allclose(x, GOLD[f"radial_fast_{n}_x"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(w, GOLD[f"radial_fast_{n}_w"], rtol=1e-14, atol=0)
    ox, ow = DO.tanh_sinh_fast(n)
    np.testing.assert_allclose(ox, x, rtol=1e-15, atol=0)
    np.testing.assert_allclose(ow, w, rtol=1e-14, atol=0)


@pytest.mark.parametrize("dm1,order", [(1, 4), (1, 6), (1, 8), (2, 4), (2, 6), (2, 8)])
def test_regular_rules_match_the_reference(dm1, order):
    x, w = TB.regular_rule(dm1, order)
    np.testing.assert_allclose(x.reshape(GOLD[f"regular_{dm1}_{order}_x"].shape),
                               GOLD[f"regular_{dm1}_{order}_x"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(w, GOLD[f"regular_{dm1}_{order}_w"], rtol=1e-14)


def test_oracle_matches_the_reference_integrator_on_golden_entries():
    from volumential_gb300.list1_gallery import generate_list1_gallery

    ints, ks, vals = GOLD["entry_ints"], GOLD["entry_k"], GOLD["entry_value"]
    worst = 0.0
    for (dim, q, kind, case, smode, tpoint, reg, rad), k, v in zip(ints, ks, vals):
        vec = generate_list1_gallery(int(dim))[0][case]
        t = DO.target_point(int(dim), int(q), 1.0, vec, int(tpoint))
        modes = np.array(np.unravel_index(int(smode), (int(q),) * int(dim)))[:, None]
        got = DO.entry_values(int(dim), int(q), 1.0, KIND[int(kind)], t[:, None], modes,
                              int(reg), int(rad), k=float(k))[0]
        worst = max(worst, abs(got - v) / abs(v))
    assert worst <= 1e-12


def test_product_entry_geometry_follows_find_target_point():
    from volumential_gb300.list1_gallery import generate_list1_gallery

    for dim, q in ((2, 3), (3, 2)):
        t = NearFieldInteractionTable(q, dim=dim, sumpy_kernel=LaplaceKernel(dim),
                                      source_box_extent=0.7)
        ids = t._get_invariant_entry_info()["entry_ids"]
        tp, dc, axes = TB.entry_geometry(t, ids)
        vecs = generate_list1_gallery(dim)[0]
        for j in np.linspace(0, len(ids) - 1, 25).astype(int):
            info = t.decode_index(ids[j])
            ref = DO.target_point(dim, q, 0.7, vecs[info["case_index"]],
                                  info["target_point_index"])
            np.testing.assert_allclose(tp[:, j], ref, rtol=1e-15, atol=1e-15)
            np.testing.assert_array_equal(
                axes[:, j], np.unravel_index(info["source_mode_index"], (q,) * dim))
        assert np.all((dc >= 0) & (dc <= 0.7))


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_constant_kernel_gives_the_exact_volume(dim):
    # test_duffy_batched_manufactured.py:129-150 (regular 6, radial 21)
    vecs = __import__("volumential_gb300.list1_gallery",
                      fromlist=["x"]).generate_list1_gallery(dim)[0]
    tps = np.stack([DO.target_point(dim, 1, 1.0, v, 0) for v in vecs], axis=1)
    vals = DO.entry_values(dim, 1, 1.0, "constant", tps, np.zeros((dim, len(vecs)), int),
                           6, 21)
    assert np.max(np.abs(vals - 1.0)) < 1e-11


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_plane_wave_matches_the_closed_form(dim):
    # test_duffy_batched_manufactured.py:219-284: cos(k x) over the unit box
    k = 1.7
    vecs = __import__("volumential_gb300.list1_gallery",
                      fromlist=["x"]).generate_list1_gallery(dim)[0]
    far = [i for i, v in enumerate(vecs) if min(v) > 0][:2]
    tps = np.stack([DO.target_point(dim, 1, 1.0, vecs[i], 0) for i in far], axis=1)
    vals = DO.entry_values(dim, 1, 1.0, "plane_wave", tps, np.zeros((dim, len(far)), int),
                           6, 21, k=k)
    x = tps[0]
    exact = (np.sin(k * (1.0 - x)) - np.sin(-k * x)) / k
    assert np.max(np.abs(vals - exact) / np.maximum(1.0, np.abs(exact))) < 1e-8


def test_duffy_order_selection_rule():
    # nearfield_potential_table.py:2576-2598: errors against the last
    # candidate, floor = the smallest positive of the (up to three) before
    # it (at least 128 eps), the first candidate within 8x the floor
    from volumential_gb300.table_builder import DEFAULT_ORDER_CANDIDATES, select_duffy_orders

    ref = np.array([1.0, -2.0, 0.5])
    errs = [1e-3, 1e-6, 1e-10, 3e-13, 2e-13, 1e-13, 0.0]
    vals = [ref + e for e in errs]
    sel, info = select_duffy_orders(DEFAULT_ORDER_CANDIDATES, vals)
    assert info["floor_estimate"] == pytest.approx(1e-13, rel=1e-3)
    assert sel == 3   # 3e-13 <= 8e-13
    # no tail to estimate from: the floor is 128 eps
    sel2, info2 = select_duffy_orders([(4, 11), (12, 61)], [ref + 1e-15, ref])
    assert info2["floor_estimate"] == 128 * np.finfo(float).eps and sel2 == 0
    # no candidate within the floor: the last one
    sel3, _ = select_duffy_orders([(4, 11), (12, 61)], [ref + 1e-3, ref])
    assert sel3 == 1
    # the floor is relative to the tail: errors 0.875, 0.375, 0.125 against
    # the last candidate give a floor of 0.125 and accept the first
    slow = [ref + e for e in (1.0, 0.5, 0.25, 0.125)]
    sel4, info4 = select_duffy_orders([(4, 11), (6, 21), (8, 31), (12, 61)], slow)
    assert info4["floor_estimate"] == 0.125 and sel4 == 0


def test_duffy_build_config_defaults():
    # nearfield_potential_table.py:195-206 and :2301-2308
    from volumential_gb300.table_builder import (
        DEFAULT_ORDER_CANDIDATES,
        DuffyBuildConfig,
        is_auto_order,
    )

    c = DuffyBuildConfig()
    assert (c.radial_rule, c.regular_quad_order, c.radial_quad_order, c.mp_dps) == (
        "tanh-sinh-fast", 20, 61, 50)
    assert (c.auto_tune_orders, c.auto_tune_samples, c.auto_tune_floor_factor,
            c.auto_tune_candidates) == (False, 5, 8.0, None)
    assert DEFAULT_ORDER_CANDIDATES[0] == (4, 11) and DEFAULT_ORDER_CANDIDATES[-1] == (12, 61)
    assert is_auto_order(None) and is_auto_order(" Auto ") and not is_auto_order(20)
