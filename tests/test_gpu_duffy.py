"""FP64 GPU table builder (``vl1_duffy_table``): entries against golden
values of the reference's own Duffy integrator and against the CPU
restatement, the reference's known answers
(``test/test_duffy_batched_manufactured.py:129-284``), and a list-1
evaluation on a table it built."""

import os

import numpy as np
import pytest

from helpers import LAP3, oracle_eval, oracle_for_workload, rel_l2
from oracle import duffy_oracle as DO
from volumential_gb300 import table_builder as TB
from volumential_gb300.kernels import ConstantKernel, HelmholtzKernel, LaplaceKernel
from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "duffy_golden.npz"))


def _table(dim, q, kind, extent=1.0):
    knl = {"laplace": LaplaceKernel(dim), "helmholtz": HelmholtzKernel(dim),
           "constant": ConstantKernel(dim), "plane_wave": LaplaceKernel(dim)}[kind]
    dt = np.complex128 if kind == "helmholtz" else np.float64
    return NearFieldInteractionTable(q, dim=dim, sumpy_kernel=knl, source_box_extent=extent,
                                     dtype=dt)


def test_gpu_entries_match_the_reference_integrator(cuda):
    ints, ks, vals = GOLD["entry_ints"], GOLD["entry_k"], GOLD["entry_value"]
    worst = 0.0
    for (dim, q, kind, case, smode, tpoint, reg, rad), k, v in zip(ints, ks, vals):
        kind = "laplace" if kind == 0 else "helmholtz"
        t = _table(int(dim), int(q), kind)
        eid = t.get_entry_index(int(smode), int(tpoint), int(case))
        _, got = TB.build_table_values(t, regular_quad_order=int(reg),
                                       radial_quad_order=int(rad), kernel=kind,
                                       k=float(k), entry_ids=[eid], store=False)
        worst = max(worst, abs(got[0] - v) / abs(v))
    assert worst <= 1e-12


@pytest.mark.parametrize("dim,q,kind", [(2, 3, "laplace"), (2, 2, "helmholtz"),
                                        (3, 2, "laplace")])
def test_gpu_table_matches_the_cpu_restatement(cuda, dim, q, kind):
    t = _table(dim, q, kind, extent=0.5)
    ids = t._get_invariant_entry_info()["entry_ids"]
    pick = ids[np.linspace(0, len(ids) - 1, 40 if dim == 2 else 12).astype(int)]
    reg, rad = (6, 21) if dim == 2 else (4, 11)
    _, got = TB.build_table_values(t, regular_quad_order=reg, radial_quad_order=rad,
                                   kernel=kind, k=4.0, entry_ids=pick, store=False)
    tp, _, axes = TB.entry_geometry(t, pick)
    ref = DO.entry_values(dim, q, 0.5, kind, tp, axes, reg, rad, k=4.0)
    assert np.max(np.abs(got - ref) / np.abs(ref)) <= 1e-12


@pytest.mark.parametrize("dim,kind,cap", [(2, "helmholtz", 3), (3, "laplace", 7)])
def test_capped_grid_gives_the_same_table_bit_for_bit(cuda, dim, kind, cap):
    # a build on a few CTAs (beside other GPU work) adds the same partial
    # sums in the same order as the one-CTA-per-item build
    t = _table(dim, 2, kind, extent=0.25)
    kw = dict(regular_quad_order=6, radial_quad_order=21, kernel=kind, k=3.0, store=False)
    ids_a, full = TB.build_table_values(t, **kw)
    ids_b, capped = TB.build_table_values(t, max_ctas=cap, **kw)
    assert np.array_equal(ids_a, ids_b)
    assert np.array_equal(np.ascontiguousarray(full).view(np.uint64),
                          np.ascontiguousarray(capped).view(np.uint64))


@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_constant_kernel_gives_the_exact_volume(cuda, dim):
    # test_duffy_batched_manufactured.py:129-150
    t = _table(dim, 1, "constant")
    t.build_table_via_duffy_radial(regular_quad_order=6, radial_quad_order=21,
                                   kernel="constant")
    ids, vals = t.get_reduced_table_data()
    assert len(ids) > 0 and t.is_built
    assert np.max(np.abs(vals - 1.0)) < 1e-11


@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_plane_wave_matches_the_closed_form(cuda, dim):
    # test_duffy_batched_manufactured.py:219-284 (cos(k x), k = 1.7)
    k = 1.7
    t = _table(dim, 1, "plane_wave")
    far = [c for c, v in enumerate(t.interaction_case_vecs) if min(v) > 0]
    ids = [t.get_entry_index(0, 0, c) for c in far]
    _, vals = TB.build_table_values(t, regular_quad_order=6, radial_quad_order=21,
                                    kernel="plane_wave", k=k, entry_ids=ids, store=False)
    x = np.array([t.find_target_point(0, c)[0] for c in far])
    exact = (np.sin(k * (1.0 - x)) - np.sin(-k * x)) / k
    assert np.max(np.abs(vals - exact) / np.maximum(1.0, np.abs(exact))) < 1e-8


def test_list1_on_a_gpu_built_laplace_table(cuda):
    """A 3D Laplace q=2 table built on the GPU, then the list-1 sum (plain and
    tensor-core paths) against the oracle on the same table."""
    import torch

    from volumential_gb300 import workloads as W
    from volumential_gb300.batch import problem_arrays
    from volumential_gb300.batched import eval_mixed

    w = W.uniform_workload("duffy3", 3, 2, 2, seed=71)
    t = _table(3, 2, "laplace", extent=w.tree.root_extent)
    t.build_table(regular_quad_order=6, radial_quad_order=21)
    assert t.is_built
    w.tables = [t]
    plan, view, keep = problem_arrays(w, cache=False)
    sh = torch.cuda.current_stream().cuda_stream
    coefs = torch.from_numpy(np.ascontiguousarray(w.coefs[0])).to("cuda")
    plain = torch.empty_like(coefs)
    mixed = torch.empty_like(coefs)
    plan.eval_fp64(view, coefs, plain, stream=sh)
    eval_mixed(plan, view, coefs, mixed, stream=sh, nrhs=1, keep=keep)
    plan.raise_on_status(sh)
    ref = oracle_eval(oracle_for_workload(w, LAP3), w, w.coefs[0])
    assert rel_l2(plain.cpu().numpy(), ref) <= 1e-12
    assert rel_l2(mixed.cpu().numpy(), ref) <= 1e-9
    plan.destroy()


def test_table_manager_builds_on_a_miss_and_reloads(cuda, tmp_path):
    from volumential_gb300.table_manager import NearFieldInteractionTableManager

    db = str(tmp_path / "cache.sqlite")
    with NearFieldInteractionTableManager(db, root_extent=1.0) as m:
        t, recomputed = m.get_table(2, "Laplace", 2, source_box_level=1,
                                    regular_quad_order=6, radial_quad_order=21)
        assert recomputed and t.is_built
        ids, vals = t.get_reduced_table_data()
    with NearFieldInteractionTableManager(db, root_extent=1.0) as m:
        t2, recomputed = m.get_table(2, "Laplace", 2, source_box_level=1)
        assert not recomputed
        ids2, vals2 = t2.get_reduced_table_data()
    np.testing.assert_array_equal(ids, ids2)
    np.testing.assert_array_equal(vals, vals2)
    # the GPU values against the CPU restatement on a few entries
    tp, _, axes = TB.entry_geometry(t, ids[:6])
    ref = DO.entry_values(2, 2, 0.5, "laplace", tp, axes, 6, 21)
    assert np.max(np.abs(vals[:6] - ref) / np.abs(ref)) <= 1e-12


def test_auto_tuned_orders_build_the_same_table_as_the_chosen_orders(cuda):
    # nearfield_potential_table.py:2465-2619 (auto_tune_orders / "auto" orders)
    from volumential_gb300.table_builder import DuffyBuildConfig

    t = _table(2, 2, "laplace", extent=0.5)
    t.build_table_via_duffy_radial(regular_quad_order="auto", radial_quad_order="auto")
    info = t.last_duffy_order_selection
    reg, rad = info["selected_regular_quad_order"], info["selected_radial_quad_order"]
    assert (reg, rad) in info["candidates"] and len(info["sample_entry_ids"]) == 5
    sel = info["candidates"].index((reg, rad))
    assert info["relative_errors_vs_best"][sel] <= info["acceptance_threshold"]
    ref = _table(2, 2, "laplace", extent=0.5)
    ref.build_table_via_duffy_radial(build_config=DuffyBuildConfig(
        regular_quad_order=reg, radial_quad_order=rad))
    a = t.get_reduced_table_data()
    b = ref.get_reduced_table_data()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
