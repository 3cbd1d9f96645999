"""Bit-exact interaction indexing, pair by pair.

For every (target box, list-1 source box) pair, the device's table key
(``vl1_classify_pairs``: table level * n_cases + case id) must equal the
oracle's, which restates the reference's FP64 case encoding
(``volumential/list1.py:439-459, 532-538, 1084-1091``: the centre difference
over the source box extent, times 4, plus shift and 1e-10, combined in base 13
and truncated after + 0.5) and its table-level rule (``list1.py:361-437``).
Trees: adaptive 2D and 3D, the C2 octree (23,087 leaves), uniform trees on a
non-dyadic root box [-0.37, 0.91]^dim, and per-level tables on an adaptive
tree.
"""

import ctypes as C

import numpy as np
import pytest

from helpers import LAP2, LAP3, MIXED_TREE_KEYS, PER_LEVEL, oracle_for_workload
from volumential_gb300 import _lib
from volumential_gb300 import workloads as W
from volumential_gb300.kernels import HelmholtzKernel, LaplaceKernel
from volumential_gb300.plan import tree_view_from_arrays

pytestmark = pytest.mark.gpu


def _device_keys(w, **wrangler_kw):
    import torch

    from helpers import wrangler_for

    wr = wrangler_for(w, **wrangler_kw)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, None)
    plan = nf.get_plan(
        table_data_combined=kw["table_data_combined"],
        mode_nmlz_combined=kw["mode_nmlz_combined"], case_indices=kw["case_indices"],
        encoding_base=kw["encoding_base"], encoding_shift=kw["encoding_shift"],
        table_root_extent=kw["table_root_extent"],
        table_starting_level=kw["table_starting_level"],
        **{n: kw[n] for n in kw if n.startswith("arithmetic_")})
    view, keep = tree_view_from_arrays(root_extent=kw["root_extent"],
                                       **{k: kw[k] for k in MIXED_TREE_KEYS})
    nnz = int(keep["lists"].numel())
    keys = torch.full((max(nnz, 1),), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.lib().vl1_classify_pairs(plan.handle, C.byref(view), keys.data_ptr(),
                                             C.c_void_p(stream)), "vl1_classify_pairs")
    st = plan.read_status(stream)
    assert st.code == _lib.VL1_OK, (st.code, st.detail0, st.detail1)
    return keys[:nnz].cpu().numpy(), plan.n_cases


def _check(w, policy, **wrangler_kw):
    keys, n_cases = _device_keys(w, **wrangler_kw)
    tr = w.traversal
    cases, levels = oracle_for_workload(w, policy).classify_pairs(
        target_boxes=tr.target_boxes,
        neighbor_source_boxes_starts=tr.neighbor_source_boxes_starts,
        neighbor_source_boxes_lists=tr.neighbor_source_boxes_lists,
        box_centers=w.tree.box_centers, box_levels=w.tree.box_levels)
    assert np.all(cases >= 0)
    expect = levels.astype(np.int64) * n_cases + cases
    assert keys.shape == expect.shape
    bad = np.flatnonzero(keys != expect)
    assert bad.size == 0, (f"{bad.size} of {keys.size} pairs differ; first at list "
                           f"position {bad[0]}: device {keys[bad[0]]}, oracle {expect[bad[0]]}")
    return keys, cases, levels


def test_adaptive_2d(cuda):
    w = W.adaptive_workload("cid2", 2, 3, tol=1e-3, max_level=7, min_level=2, seed=401,
                            n_terms=8, width_range=(0.02, 0.1))
    _, cases, _ = _check(w, LAP2)
    assert len(np.unique(cases)) == 33   # every 2D case (2:1 levels included) occurs


def test_adaptive_3d(cuda):
    w = W.adaptive_workload("cid3", 3, 2, tol=3e-2, max_level=5, min_level=2, seed=402)
    _, cases, _ = _check(w, LAP3)
    assert len(np.unique(cases)) > 100


def test_c2_octree(cuda):
    w = W.config_c2(tables="synthetic")
    keys, cases, _ = _check(w, LAP3)
    assert keys.size == 565335


@pytest.mark.parametrize("dim,level", [(2, 5), (3, 3)])
def test_uniform_non_dyadic_root_box(cuda, dim, level):
    w = W.uniform_workload("cid_nd", dim, level, 2, seed=403, a=-0.37, b=0.91)
    assert w.tree.root_extent == pytest.approx(1.28)
    _check(w, LAP2 if dim == 2 else LAP3)


def test_adaptive_non_dyadic_root_box(cuda):
    from volumential_gb300.tree_build import build_adaptive_tree, build_list1_traversal

    mix = W.random_gaussian_mixture(np.random.default_rng(404), 2, 6, (0.02, 0.1),
                                    a=-0.37, b=0.91)

    def refine(nodes):
        v = mix(nodes)
        return (v.max(axis=-1) - v.min(axis=-1)) > 1e-3

    tree = build_adaptive_tree(2, 2, refine, max_level=7, min_level=2, a=-0.37, b=0.91)
    trav = build_list1_traversal(tree)
    w = W.Workload("cid_adnd", 2, 2, LaplaceKernel(2), trav,
                   W.synthetic_tables(2, 2, LaplaceKernel(2), source_box_extent=1.28),
                   mix(tree.targets)[None, :], 404)
    _check(w, LAP2)


def test_per_level_tables_on_adaptive_tree(cuda):
    w = W.adaptive_workload("cid_pl", 2, 2, tol=1e-3, max_level=7, min_level=2, seed=405,
                            n_terms=8, width_range=(0.02, 0.1), kernel=HelmholtzKernel(2))
    lv = w.tree.box_levels[w.traversal.target_boxes]
    lo, hi = int(lv.min()), int(lv.max())
    # tables for levels lo + 1 .. hi - 1: source boxes of level lo lie below
    # the first table and those of level hi beyond the last, so both clamps
    # of the level rule occur
    w.tables = W.synthetic_tables(2, 2, w.kernel, n_tables=hi - lo - 1, seed=9,
                                  complex_values=True,
                                  source_box_extent=w.tree.root_extent / 2 ** (lo + 1))
    _, _, levels = _check(w, PER_LEVEL)
    assert levels.min() == 0 and levels.max() == hi - lo - 2
