"""GPU parity on physical tables: the tables the benchmark configurations name,
built by the FP64 GPU Duffy builder at the reference's default orders
(regular 20, radial 61, tanh-sinh-fast), fed to both GPU paths and to the C
oracle, on reduced trees of the same dimension and q:

* 2D Laplace q=4, canonical table (level 0, inferred scaling, log term) --
  the table of config 1;
* 3D Laplace q=4, canonical table (scaling h_s^2 / h_0^2) -- config 2;
* 2D Helmholtz k=20 q=5, one fixed complex table at source box extent 1/64
  (a level-6 box of the unit square) -- config 3.

Physical tables span a wide range of magnitudes (log-singular self cases next
to small far entries), which the mixed path's fixed-point digits must carry:
the plain FP64 path must match the oracle within 1e-12 relative l2 and the
tensor-core path within 1e-9, for every right-hand side.
"""

import numpy as np
import pytest

from helpers import FIXED, LAP2, LAP3, oracle_eval, oracle_for_workload, rel_l2, wrangler_for
from volumential_gb300 import workloads as W
from volumential_gb300.kernels import HelmholtzKernel

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_MIXED = 1e-9


def _both_paths(w, policy):
    """Per-rhs relative l2 errors of the plain and mixed paths vs the oracle."""
    wr = wrangler_for(w)
    tr = w.traversal
    args = (tr.target_boxes, tr.neighbor_source_boxes_starts, tr.neighbor_source_boxes_lists,
            w.coefs)
    plain = wr.eval_direct_batched(*args)[0][0].cpu().numpy()
    mixed = wr.eval_direct_batched(*args, precision="mixed")[0][0].cpu().numpy()
    prob = oracle_for_workload(w, policy)
    e_plain, e_mixed = [], []
    for r in range(w.nrhs):
        ref = oracle_eval(prob, w, w.coefs[r])
        assert np.linalg.norm(ref) > 0
        e_plain.append(rel_l2(plain[r], ref))
        e_mixed.append(rel_l2(mixed[r], ref))
    print(f"{w.name}: plain max {max(e_plain):.2e}, mixed per rhs "
          + " ".join(f"{e:.2e}" for e in e_mixed))
    assert max(e_plain) <= TOL_FP64, e_plain
    assert max(e_mixed) <= TOL_MIXED, e_mixed
    return e_plain, e_mixed


def _table_range(w):
    vals = np.abs(np.asarray(w.tables[0].get_reduced_table_data()[1]))
    vals = vals[vals > 0]
    return float(vals.max() / vals.min())


def test_2d_laplace_q4_duffy_table_uniform(cuda):
    w = W.uniform_workload("phys_lap2d_u4", 2, 4, 4, seed=301, nrhs=3, tables="duffy")
    assert _table_range(w) > 10.0   # a physical table, not seeded noise
    _both_paths(w, LAP2)


def test_2d_laplace_q4_duffy_table_adaptive(cuda):
    w = W.adaptive_workload("phys_lap2d_ad", 2, 4, tol=1e-3, max_level=7, min_level=2,
                            seed=302, n_terms=8, width_range=(0.02, 0.1), nrhs=2,
                            tables="duffy")
    assert len(np.unique(w.tree.box_levels[w.traversal.target_boxes])) > 2
    _both_paths(w, LAP2)


def test_3d_laplace_q4_duffy_table_adaptive(cuda):
    w = W.adaptive_workload("phys_lap3d_ad", 3, 4, tol=3e-2, max_level=5, min_level=2,
                            seed=303, nrhs=2, tables="duffy")
    assert len(np.unique(w.tree.box_levels[w.traversal.target_boxes])) > 1
    assert _table_range(w) > 10.0
    _both_paths(w, LAP3)


def test_3d_laplace_q4_duffy_table_uniform(cuda):
    w = W.uniform_workload("phys_lap3d_u3", 3, 3, 4, seed=304, nrhs=1, tables="duffy",
                           n_terms=16, width_range=(0.01, 0.08))
    _both_paths(w, LAP3)


def test_2d_helmholtz_k20_q5_duffy_fixed_table(cuda):
    # leaves of extent 1/64, as the level-6 boxes of config 3: a level-3 tree
    # on a square of side 1/8
    w = W.uniform_workload("phys_helm2d", 2, 3, 5, seed=305, nrhs=4,
                           kernel=HelmholtzKernel(2), complex_table=True,
                           a=-1.0 / 16, b=1.0 / 16, width_range=(0.005, 0.02))
    w.tables = W.duffy_tables(2, 5, w.kernel, source_box_extent=1.0 / 64, k=20.0,
                              complex_values=True)
    assert w.tables[0].source_box_extent == w.tree.root_extent / 8
    _both_paths(w, FIXED)
