"""GPU parity of the mixed-precision (tensor-core) list-1 path.

The mixed path must match the FP64 oracle within 1e-9 relative l2 (the
mixed-precision tolerance); its error model is ~2^-40 of sum |table||density|,
so the measured errors are expected near 1e-12.
"""

import numpy as np
import pytest

from helpers import FIXED, LAP2, LAP3, oracle_eval, oracle_for_workload, rel_l2, wrangler_for
from volumential_gb300 import workloads as W
from volumential_gb300.kernels import HelmholtzKernel

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-9


def _mixed(w, coefs=None):
    wr = wrangler_for(w)
    tr = w.traversal
    c = w.coefs if coefs is None else coefs
    outs, _ = wr.eval_direct_batched(tr.target_boxes, tr.neighbor_source_boxes_starts,
                                     tr.neighbor_source_boxes_lists, c, precision="mixed")
    return outs[0].cpu().numpy()


def _check(w, policy, coefs=None, tol=TOL_MIXED):
    prob = oracle_for_workload(w, policy)
    c = w.coefs if coefs is None else coefs
    got = _mixed(w, c)
    errs = []
    for r in range(c.shape[0]):
        ref = oracle_eval(prob, w, c[r])
        errs.append(rel_l2(got[r], ref))
    assert max(errs) <= tol, errs
    return max(errs)


def test_mixed_2d_laplace_uniform_q4(cuda):
    err = _check(W.uniform_workload("m2", 2, 4, 4, seed=31), LAP2)
    print("rel l2", err)


def test_mixed_2d_laplace_q3_small_k(cuda):
    _check(W.uniform_workload("m3", 2, 3, 3, seed=32), LAP2)


def test_mixed_3d_laplace_adaptive_q4(cuda):
    w = W.adaptive_workload("ma3", 3, 4, tol=3e-2, max_level=5, min_level=2, seed=33)
    _check(w, LAP3)


def test_mixed_3d_q5_two_k_chunks(cuda):
    _check(W.uniform_workload("m5", 3, 2, 5, seed=34), LAP3)


def test_mixed_2d_helmholtz_complex_table(cuda):
    w = W.uniform_workload("mh", 2, 4, 5, seed=35, kernel=HelmholtzKernel(2),
                           complex_table=True, nrhs=3)
    w.tables = W.synthetic_tables(2, 5, w.kernel, seed=6, complex_values=True,
                                  source_box_extent=w.tree.root_extent / 16)
    _check(w, FIXED)


def test_mixed_many_rhs_spanning_tiles(cuda):
    w = W.uniform_workload("mr", 2, 3, 4, seed=36, nrhs=130)
    _check(w, LAP2)


def test_mixed_complex_coefficients(cuda):
    w = W.uniform_workload("mc", 2, 3, 3, seed=37, nrhs=2)
    c = w.coefs + 1j * w.coefs[::-1]
    _check(w, LAP2, coefs=c)


def test_mixed_zero_density_rhs(cuda):
    w = W.uniform_workload("mz", 2, 3, 3, seed=38, nrhs=2)
    c = w.coefs.copy()
    c[1] = 0.0
    got = _mixed(w, c)
    assert np.all(got[1] == 0.0)
    prob = oracle_for_workload(w, LAP2)
    assert rel_l2(got[0], oracle_eval(prob, w, c[0])) <= TOL_MIXED


def test_mixed_matches_plain_fp64_on_config1(cuda):
    w = W.config_c1(seed=39)
    wr = wrangler_for(w)
    tr = w.traversal
    plain, _ = wr.eval_direct_batched(tr.target_boxes, tr.neighbor_source_boxes_starts,
                                      tr.neighbor_source_boxes_lists, w.coefs)
    mixed, _ = wr.eval_direct_batched(tr.target_boxes, tr.neighbor_source_boxes_starts,
                                      tr.neighbor_source_boxes_lists, w.coefs,
                                      precision="mixed")
    assert rel_l2(mixed[0].cpu().numpy(), plain[0].cpu().numpy()) <= TOL_MIXED


def test_mixed_2d_q9_k_padded_to_rounds(cuda):
    # 81 modes: K pads to 128 (two exact rounds of two 32-wide chunks)
    _check(W.uniform_workload("m9", 2, 3, 9, seed=39), LAP2)
