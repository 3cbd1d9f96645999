"""Helmholtz split mode on the GPU: the list-1 remainder sum
(``vl1_split_correction``) against the CPU restatement
(``oracle/split_oracle.py``, closed-form remainder), and the whole split
evaluation (Laplace table + remainder, through ``drive_volume_fmm``) against
the list-1 sum with a Helmholtz table built for the same tree, which it must
approximate to the quadrature error of the smooth remainder."""

import numpy as np
import pytest

from helpers import rel_l2
from oracle import split_oracle as SO
from volumential_gb300 import workloads as W
from volumential_gb300.expansion_wrangler_fpnd import (
    FPNDExpansionWrangler,
    FPNDTreeIndependentDataForWrangler,
)
from volumential_gb300.helmholtz_split import max_neighbor_distance, series_terms
from volumential_gb300.kernels import HelmholtzKernel, LaplaceKernel
from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable
from volumential_gb300.volume_fmm import drive_volume_fmm

pytestmark = pytest.mark.gpu


# real wave numbers take the kernel's two-sum form of the series, complex ones
# the general four-sum form
@pytest.mark.parametrize("dim,level,q,k", [(2, 3, 3, 20.0), (3, 2, 2, 5.0 + 0.3j),
                                           (3, 2, 3, 7.0), (2, 3, 3, 12.0 + 0.5j)])
@pytest.mark.parametrize("exclude_self", [True, False])
def test_remainder_sum_matches_the_closed_form_restatement(cuda, dim, level, q, k,
                                                           exclude_self):
    import torch

    from volumential_gb300.batch import tree_arrays
    from volumential_gb300.helmholtz_split import split_correction

    w = W.uniform_workload("split", dim, level, q, seed=91, kernel=HelmholtzKernel(dim))
    tree, tr = w.tree, w.traversal
    view, keep = tree_arrays(w)
    rng = np.random.default_rng(3)
    wts = rng.standard_normal(tree.ntargets) + (1j * rng.standard_normal(tree.ntargets)
                                               if dim == 3 else 0.0)
    pts = torch.from_numpy(np.ascontiguousarray(tree.targets)).to("cuda")
    n = series_terms(dim, k, max_neighbor_distance(tree))
    got = split_correction(view, pts, torch.from_numpy(np.asarray(wts)).to("cuda"), k, n,
                           exclude_self=exclude_self).cpu().numpy()
    ref = SO.split_sum(dim, k, tree.targets, np.asarray(wts, dtype=np.complex128),
                       tr.target_boxes, tr.neighbor_source_boxes_starts,
                       tr.neighbor_source_boxes_lists, tree.box_target_starts,
                       tree.box_target_counts_nonchild, exclude_self=exclude_self)
    assert rel_l2(got, ref) <= 1e-12


def test_split_mode_approximates_the_helmholtz_table(cuda):
    import torch

    k = 20.0
    w = W.uniform_workload("split2d", 2, 4, 4, seed=92, kernel=HelmholtzKernel(2))
    tree, trav = w.tree, w.traversal
    lap = NearFieldInteractionTable(4, dim=2, sumpy_kernel=LaplaceKernel(2),
                                    source_box_extent=tree.root_extent)
    lap.build_table(regular_quad_order=8, radial_quad_order=31)
    helm = NearFieldInteractionTable(4, dim=2, sumpy_kernel=HelmholtzKernel(2),
                                     source_box_extent=tree.root_extent / 16,
                                     dtype=np.complex128)
    helm.build_table(regular_quad_order=8, radial_quad_order=31, k=k)
    ti = FPNDTreeIndependentDataForWrangler(target_kernels=[HelmholtzKernel(2)])
    dens = w.coefs[0]
    weights = dens * tree.weights
    ws = FPNDExpansionWrangler(ti, trav, [lap], dtype=np.complex128, quad_order=4,
                               kernel_extra_kwargs={"k": k})
    assert ws.helmholtz_split
    wh = FPNDExpansionWrangler(ti, trav, [helm], dtype=np.complex128, quad_order=4,
                               kernel_extra_kwargs={"k": k})
    assert not wh.helmholtz_split
    ps = drive_volume_fmm(trav, ws, weights, dens, list1_only=True, reorder_sources=False,
                          reorder_potentials=False)
    ph = drive_volume_fmm(trav, wh, weights, dens, list1_only=True, reorder_sources=False,
                          reorder_potentials=False)
    a = ps[0].cpu().numpy() if hasattr(ps[0], "cpu") else np.asarray(ps[0])
    b = ph[0].cpu().numpy() if hasattr(ph[0], "cpu") else np.asarray(ph[0])
    err = rel_l2(a, b)
    assert np.all(np.isfinite(a)) and err <= 1e-4, err
    # without the remainder the Laplace part alone is far off
    lap_only, _ = ws.eval_direct(trav.target_boxes, trav.neighbor_source_boxes_starts,
                                 trav.neighbor_source_boxes_lists, dens)
    assert rel_l2(lap_only[0].cpu().numpy(), b) > 100 * err
    torch.cuda.synchronize()
