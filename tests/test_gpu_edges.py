"""Edge cases of the list-1 path on the GPU: an empty target set, a tree of
one box, densities whose magnitude varies over hundreds of decades across the
domain (the FP64 path keeps every box's relative accuracy, the tensor-core
path its bound relative to the rhs's largest value) or sits near the bottom
of the FP64 range."""

import numpy as np
import pytest

from helpers import LAP2, LAP3, oracle_eval, oracle_for_workload, rel_l2, wrangler_for
from volumential_gb300 import workloads as W
from volumential_gb300.tree_build import Traversal, build_list1_traversal, build_uniform_tree

pytestmark = pytest.mark.gpu


def _eval(w, coefs, precision):
    import torch

    wr = wrangler_for(w)
    tr = w.traversal
    outs, _ = wr.eval_direct_batched(tr.target_boxes, tr.neighbor_source_boxes_starts,
                                     tr.neighbor_source_boxes_lists,
                                     np.ascontiguousarray(coefs)[None, :], precision=precision)
    torch.cuda.synchronize()
    return outs[0][0].cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_target_set_writes_nothing(cuda, precision):
    import torch

    w = W.uniform_workload("edge_empty", 2, 2, 3, seed=5)
    tr = w.traversal
    wr = wrangler_for(w)
    empty = np.zeros(0, dtype=np.int32)
    nf_out = torch.full((w.n_points,), 7.0, dtype=torch.float64, device="cuda")
    pots, _ = wr.eval_direct(empty, np.zeros(1, dtype=np.int32), empty, w.coefs[0])
    assert np.all(pots[0].cpu().numpy() == 0.0)      # output_zeros, untouched
    outs, _ = wr.eval_direct_batched(empty, np.zeros(1, dtype=np.int32), empty,
                                     w.coefs[:1], precision=precision)
    assert outs[0].shape == (1, w.n_points)
    assert nf_out[0].item() == 7.0


@pytest.mark.parametrize("dim,policy", [(2, LAP2), (3, LAP3)])
def test_single_box_tree(cuda, dim, policy):
    tree = build_uniform_tree(dim, 0, 3)
    trav = build_list1_traversal(tree)
    np.testing.assert_array_equal(trav.neighbor_source_boxes_lists, [0])
    w = W.uniform_workload("edge_one", dim, 0, 3, seed=6)
    ref = oracle_eval(oracle_for_workload(w, policy), w, w.coefs[0])
    assert rel_l2(_eval(w, w.coefs[0], "fp64"), ref) <= 1e-12
    assert rel_l2(_eval(w, w.coefs[0], "mixed"), ref) <= 1e-9


@pytest.mark.parametrize("dim,policy", [(2, LAP2), (3, LAP3)])
def test_densities_over_hundreds_of_decades(cuda, dim, policy):
    # scale 10^(250 sin(2 pi x)): smooth in space, so each target's list-1
    # neighbourhood has a similar scale while the domain spans ~500 decades.
    # The FP64 path keeps every box's relative accuracy; the tensor-core path
    # writes the densities of an rhs against one scale (its largest value),
    # so its error is bounded relative to the largest output, and boxes many
    # decades below it come out as (near) zero.
    w = W.uniform_workload("edge_scale", dim, 3 if dim == 2 else 2, 3, seed=7)
    x = w.tree.targets[0]
    coefs = w.coefs[0] * 10.0 ** (250.0 * np.sin(2 * np.pi * x))
    ref = oracle_eval(oracle_for_workload(w, policy), w, coefs)
    plain = _eval(w, coefs, "fp64")
    mixed = _eval(w, coefs, "mixed")
    assert np.all(np.isfinite(plain)) and np.all(np.isfinite(mixed))
    # relative error per target box, against that box's own scale
    tr = w.traversal
    starts, counts = w.tree.box_target_starts, w.tree.box_target_counts_nonchild
    worst_p = 0.0
    for tb in tr.target_boxes:
        sl = slice(starts[tb], starts[tb] + counts[tb])
        scale = np.max(np.abs(ref[sl]))
        if scale == 0:
            continue
        worst_p = max(worst_p, np.max(np.abs(plain[sl] - ref[sl])) / scale)
    assert worst_p <= 1e-11
    s = np.max(np.abs(ref))   # norms of values near 1e250 would overflow
    assert rel_l2(mixed / s, ref / s) <= 1e-9
    assert np.max(np.abs(mixed - ref)) <= 1e-9 * s


def test_densities_near_the_bottom_of_fp64(cuda):
    w = W.uniform_workload("edge_tiny", 3, 2, 3, seed=8)
    coefs = w.coefs[0] * 1e-300
    ref = oracle_eval(oracle_for_workload(w, LAP3), w, coefs)
    mixed = _eval(w, coefs, "mixed")
    assert np.all(np.isfinite(mixed)) and np.max(np.abs(mixed)) > 0
    assert rel_l2(mixed, ref) <= 1e-9


def test_tree_view_cache_follows_in_place_changes(cuda):
    """Repeated calls over one set of CUDA tree tensors reuse the tree view;
    an in-place change of any of them (its version counter) rebuilds and
    revalidates it, so a bad index written into a cached tree still raises."""
    import torch

    from volumential_gb300.plan import tree_view_from_arrays

    w = W.uniform_workload("edge_viewcache", 2, 2, 3, seed=9)
    tr, tree = w.traversal, w.tree
    local = tree.box_local_mode_ids()
    dev = lambda a, dt=torch.int32: torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dt)
    arrays = dict(
        target_boxes=dev(tr.target_boxes), neighbor_source_boxes_starts=dev(tr.neighbor_source_boxes_starts),
        neighbor_source_boxes_lists=dev(tr.neighbor_source_boxes_lists),
        box_centers=dev(tree.box_centers, torch.float64), box_levels=dev(tree.box_levels, torch.uint8),
        box_source_starts=dev(tree.box_target_starts),
        box_source_counts_nonchild=dev(tree.box_target_counts_nonchild),
        box_target_starts=dev(tree.box_target_starts),
        box_target_counts_nonchild=dev(tree.box_target_counts_nonchild),
        source_mode_ids=dev(local), target_point_ids=dev(local), root_extent=tree.root_extent)
    v1, k1 = tree_view_from_arrays(**arrays)
    v2, k2 = tree_view_from_arrays(**arrays)
    assert v2 is v1 and k2 is k1
    lists = arrays["neighbor_source_boxes_lists"]
    lists[0] = lists[0]                      # same value, new version
    v3, _ = tree_view_from_arrays(**arrays)
    assert v3 is not v1
    lists[0] = int(tree.box_levels.size) + 5  # a source box past the tree
    with pytest.raises(ValueError):
        tree_view_from_arrays(**arrays)
