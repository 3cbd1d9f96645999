"""Batches of problems evaluated by one persistent tensor-core launch per
kernel shape (``vl1_batch_create`` / ``vl1_batch_eval``).

Each problem's result must be identical, bit for bit, to its own
``vl1_eval_mixed`` evaluation with the same schedule (the batch runs the same
work items and the same arithmetic), match the FP64 oracle within the mixed
tolerance, and a CUDA-graph replay must follow the coefficients it is given.
"""

import numpy as np
import pytest

from helpers import FIXED, LAP2, LAP3, oracle_eval, oracle_for_workload, rel_l2
from volumential_gb300 import workloads as W
from volumential_gb300.batch import BatchProblem, MixedBatch, autotune_batch, problem_arrays
from volumential_gb300.batched import eval_mixed
from volumential_gb300.kernels import HelmholtzKernel
from volumential_gb300.plan import as_device_tensor

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-9


def _workloads():
    ws = [
        (W.uniform_workload("b3q3", 3, 2, 3, seed=61, nrhs=2), LAP3),
        (W.uniform_workload("b3q4", 3, 2, 4, seed=62, nrhs=1), LAP3),
        (W.uniform_workload("b3q5", 3, 2, 5, seed=63, nrhs=3), LAP3),   # two column chunks
        (W.adaptive_workload("b3ad", 3, 4, tol=3e-2, max_level=5, min_level=2, seed=64,
                             nrhs=2), LAP3),
        (W.uniform_workload("b2q4", 2, 4, 4, seed=65, nrhs=2), LAP2),   # K chunk 16, log term
    ]
    h = W.uniform_workload("b2h", 2, 3, 5, seed=66, kernel=HelmholtzKernel(2),
                           complex_table=True, nrhs=2)
    h.tables = W.synthetic_tables(2, 5, h.kernel, seed=8, complex_values=True,
                                  source_box_extent=h.tree.root_extent / 8)
    ws.append((h, FIXED))
    return ws


def _problems(torch, ws):
    probs = []
    for w, _ in ws:
        plan, view, keep = problem_arrays(w)
        coefs = as_device_tensor(np.ascontiguousarray(w.coefs))
        odt = torch.complex128 if plan.complex_table else torch.float64
        out = torch.full((w.nrhs, w.n_points), float("nan"), dtype=odt, device="cuda")
        probs.append(BatchProblem(plan, view, keep, coefs, out, w.nrhs))
    return probs


def _singles(torch, probs, cap):
    sh = torch.cuda.current_stream().cuda_stream
    outs = []
    for p in probs:
        o = torch.full_like(p.out, float("nan"))
        eval_mixed(p.plan, p.view, p.coefs, o, stream=sh, nrhs=p.nrhs, keep=p.keep,
                   max_keys_per_item=cap)
        outs.append(o.cpu().numpy())
    return outs


@pytest.mark.parametrize("cap", [None, 2])
def test_batch_matches_single_problem_evaluations_bitwise(cuda, cap):
    torch = cuda
    ws = _workloads()
    probs = _problems(torch, ws)
    batch = MixedBatch(probs, max_keys_per_item=cap)
    assert len({(p.plan.mixed_geometry()["nch"], p.plan.mixed_geometry()["kc"])
                for p in probs}) >= 2
    batch.eval()
    batch.raise_on_status()
    singles = _singles(torch, probs, cap)
    for p, ref in zip(probs, singles):
        got = p.out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.array_equal(got, ref)
    for (w, pol), p in zip(ws, probs):
        prob = oracle_for_workload(w, pol)
        got = p.out.cpu().numpy()
        for r in range(w.nrhs):
            assert rel_l2(got[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED
    batch.close()


def test_batch_graph_replay_follows_the_coefficients(cuda):
    torch = cuda
    ws = _workloads()[:4]
    probs = _problems(torch, ws)
    batch = MixedBatch(probs, ctas_per_launch=37)
    batch.capture()
    batch.replay()
    torch.cuda.synchronize()
    first = [p.out.cpu().numpy().copy() for p in probs]
    for p in probs:
        p.coefs.mul_(2.0)                    # powers of two scale the results exactly
        p.out.fill_(float("nan"))
    batch.replay()
    torch.cuda.synchronize()
    batch.raise_on_status()
    for p, f in zip(probs, first):
        assert np.array_equal(p.out.cpu().numpy(), 2.0 * f)
    batch.close()


def _default_shapes(probs):
    return {id(p.plan): (p.plan, p.plan.mixed_geometry()) for p in probs}


def _restore(saved):
    for plan, geo in saved.values():
        plan.set_mixed_geometry(geo["kc"], geo["nch"])


def test_autotuned_batch_gives_the_same_results(cuda):
    torch = cuda
    ws = _workloads()[:3]
    probs = _problems(torch, ws)
    saved = _default_shapes(probs)
    try:
        batch, table = autotune_batch(probs, reps=1, divisors=(1, 4))
        batch.eval()
        batch.raise_on_status()
        # every plan's shapes were timed and one chosen
        labels = {f"3d_q{q}" for q in (3, 4, 5)}
        assert set(table["shapes"]) == labels
        for rows in table["shapes"].values():
            assert rows["chosen"] in rows and len(rows) >= 3
        for (w, pol), p in zip(ws, probs):
            prob = oracle_for_workload(w, pol)
            got = p.out.cpu().numpy()
            for r in range(w.nrhs):
                assert rel_l2(got[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED
        batch.close()
    finally:
        _restore(saved)


@pytest.mark.parametrize("kc,nch", [(16, 16), (16, 32), (16, 64), (32, 16), (32, 32),
                                    (32, 64)])
def test_every_tile_shape_matches_the_oracle(cuda, kc, nch):
    """Each tensor-core kernel instance (K chunk x column chunk) on a 3D q=4
    adaptive tree and a 2D complex-table problem, single calls and a batch."""
    torch = cuda
    ws = [(W.adaptive_workload("shape3", 3, 4, tol=3e-2, max_level=4, min_level=2, seed=67,
                               nrhs=2), LAP3)]
    h = W.uniform_workload("shape_h", 2, 3, 5, seed=68, kernel=HelmholtzKernel(2),
                           complex_table=True, nrhs=1)
    h.tables = W.synthetic_tables(2, 5, h.kernel, seed=9, complex_values=True,
                                  source_box_extent=h.tree.root_extent / 8)
    ws.append((h, FIXED))
    probs = _problems(torch, ws)
    saved = _default_shapes(probs)
    try:
        for p in probs:
            p.plan.set_mixed_geometry(kc, nch)
            assert (p.plan.mixed_geometry()["kc"], p.plan.mixed_geometry()["nch"]) == (kc, nch)
        singles = _singles(torch, probs, None)
        batch = MixedBatch(probs)
        batch.eval()
        batch.raise_on_status()
        for (w, pol), p, single in zip(ws, probs, singles):
            prob = oracle_for_workload(w, pol)
            got = p.out.cpu().numpy()
            assert np.array_equal(got, single)
            for r in range(w.nrhs):
                assert rel_l2(got[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_MIXED
        batch.close()
    finally:
        _restore(saved)
