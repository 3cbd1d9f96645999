"""Serving (``volumential_gb300.serving``): continuous batching of single-rhs
requests over resident plans and trees.

Each request's result must be bit-identical whether it is evaluated alone or
in a step with other requests (its work items and arithmetic do not depend
on the mix), match the FP64 oracle within the mixed tolerance, and stay the
same when a small HBM budget forces residents to be evicted and rebuilt.
"""

import numpy as np
import pytest

from helpers import LAP2, LAP3, PER_LEVEL, oracle_eval, oracle_for_workload, rel_l2
from volumential_gb300 import workloads as W
from volumential_gb300.serving import AdmissionError, ServingEngine

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-9


def _mix():
    probs, reqs, mixes = W.config_c5(seed=5100, n_requests=48, n_range=(1e3, 3e4))
    ws = W.c5_workloads(probs, seed=5100)
    return probs, reqs, mixes, ws


def _engine(ws, **kw):
    eng = ServingEngine(**kw)
    for key, w in ws.items():
        eng.register(key, w, w.meta["table_key"], w.meta["tree_key"], w.meta["sched_key"])
    return eng


def _densities(torch, ws, mixes):
    dens = {}
    for key, w in ws.items():
        pts = torch.from_numpy(np.ascontiguousarray(w.tree.targets)).to("cuda")
        dens[key] = [m.on_device(pts).contiguous() for m in mixes[key]]
    return dens


def _policy(w):
    if w.kernel.is_complex_valued:
        return PER_LEVEL
    return LAP2 if w.dim == 2 else LAP3


def _chosen(probs):
    """One problem of each (dim, kernel)."""
    seen, out = set(), []
    for key in sorted(probs):
        if (key[0], key[1]) not in seen:
            seen.add((key[0], key[1]))
            out.append(key)
    return out


def test_serving_results_are_the_same_alone_and_in_the_mix(cuda):
    torch = cuda
    probs, reqs, mixes, ws = _mix()
    dens = _densities(torch, ws, mixes)
    eng = _engine(ws, hbm_budget_bytes=8 << 30, step_capacity_bytes=256 << 20,
                  max_step_requests=16)
    chosen = _chosen(probs)
    assert len(chosen) == 4
    alone = {}
    for key in chosen:
        r = eng.submit(key, dens[key][0])
        eng.drain()
        assert eng.step_sizes[-1] == 1
        alone[key] = r.out.cpu().numpy()
    # the whole mix at once (several steps of up to 16), the chosen problems
    # again in the middle of it
    mixed = {}
    for i, (key, di) in enumerate(reqs):
        eng.submit(key, dens[key][di])
        if i == len(reqs) // 2:
            for k in chosen:
                mixed[k] = eng.submit(k, dens[k][0])
    done = eng.drain()
    eng.check_status()
    assert len(done) == len(reqs) + len(chosen)
    assert max(eng.step_sizes) == 16
    for key in chosen:
        got = mixed[key].out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.array_equal(got, alone[key]), key
        w = ws[key]
        ref = oracle_eval(oracle_for_workload(w, _policy(w)), w,
                          dens[key][0].cpu().numpy())
        assert rel_l2(got, ref) <= TOL_MIXED, key
    # every request of the mix against the oracle on a sample
    sample = [q for q in done if q.key not in alone][:12]
    for q in sample:
        w = ws[q.key]
        ref = oracle_eval(oracle_for_workload(w, _policy(w)), w, q.coefs.cpu().numpy())
        assert rel_l2(q.out.cpu().numpy(), ref) <= TOL_MIXED, q.key
    eng.close()


def test_serving_under_a_small_budget_evicts_and_rebuilds(cuda):
    torch = cuda
    probs, reqs, mixes, ws = _mix()
    dens = _densities(torch, ws, mixes)
    keys = sorted(probs)[:6]
    big = _engine(ws, hbm_budget_bytes=8 << 30, step_capacity_bytes=64 << 20)
    ref = {}
    for k in keys:
        ref[k] = big.submit(k, dens[k][1])
    big.drain()
    big.close()
    # the largest plan + tree + schedule of the six fits, all six do not
    need = {}
    for k in keys:
        e = _engine(ws, hbm_budget_bytes=8 << 30, step_capacity_bytes=64 << 20)
        e.submit(k, dens[k][1])
        e.drain()
        need[k] = e.budget.used          # plan, tree, schedule and one request slot
        e.close()
    budget = max(need.values()) + 4096
    assert sum(need.values()) > budget
    small = _engine(ws, hbm_budget_bytes=budget, step_capacity_bytes=64 << 20,
                    max_step_requests=1)
    for _ in range(2):
        for k in keys:
            r = small.submit(k, dens[k][1])
            small.drain()
            assert small.budget.used <= budget
            assert np.array_equal(r.out.cpu().numpy(), ref[k].out.cpu().numpy()), k
    assert small.budget.evictions > 0
    small.check_status()
    small.close()
    tiny = _engine(ws, hbm_budget_bytes=1 << 10, step_capacity_bytes=64 << 20)
    with pytest.raises(AdmissionError):
        tiny.admit(keys[0])
    tiny.close()


def test_tables_built_on_arrival_do_not_stall_the_other_problems(cuda):
    """A Helmholtz problem with a real wave number arrives without tables:
    its first request starts the FP64 Duffy build on the engine's build
    thread; requests of resident problems submitted after it complete while
    the build runs (the build function holds an event the test sets only
    once they are done), the new problem's requests are served once the
    table exists, and its results match the oracle on that table and are the
    same bits alone and in the mix."""
    import threading

    torch = cuda
    probs, reqs, mixes, ws = _mix()
    dens = _densities(torch, ws, mixes)
    new = W.config_c5_arrivals(seed=5600, n_new=1, n_range=(1e3, 3e3), qs=(3,))
    new_ws, builders = W.c5_arrival_workloads(new)
    (nkey, nw), = new_ws.items()
    assert nkey[2] != int(nkey[2])          # a real wave number
    release = threading.Event()

    def build():
        assert release.wait(60.0)
        return builders[nkey]()

    eng = _engine(ws, hbm_budget_bytes=8 << 30, step_capacity_bytes=256 << 20,
                  max_step_requests=8)
    eng.register(nkey, nw, nw.meta["table_key"], nw.meta["tree_key"], nw.meta["sched_key"],
                 build_tables=build)
    pts = torch.from_numpy(np.ascontiguousarray(nw.tree.targets)).to("cuda")
    rng = np.random.default_rng(3)
    x = W.random_gaussian_mixture(rng, nw.dim, 6, (0.05, 0.2)).on_device(pts).contiguous()
    first = eng.submit(nkey, x)
    assert first.waited_build
    others = [eng.submit(k, dens[k][di]) for k, di in reqs[:24]]
    while any(q.t_done is None for q in others):
        eng.pump()
    assert first.t_done is None and eng.table_builds == 0
    release.set()
    eng.drain()
    assert first.t_done is not None and eng.table_builds == 1
    eng.check_status()
    got = first.out.cpu().numpy()
    alone = eng.submit(nkey, x)
    eng.drain()
    assert np.array_equal(alone.out.cpu().numpy(), got)
    tables = eng._tables[nw.meta["table_key"]]
    built = W.Workload(nw.name, nw.dim, nw.q, nw.kernel, nw.traversal, tables,
                       np.zeros((1, 0)), nw.seed, meta=nw.meta)
    ref = oracle_eval(oracle_for_workload(built, PER_LEVEL), built, x.cpu().numpy())
    assert rel_l2(got, ref) <= TOL_MIXED
    eng.close()
