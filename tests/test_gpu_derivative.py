"""Derivative-kernel tables (AxisTargetDerivative / AxisSourceDerivative of
Laplace and Helmholtz) from the FP64 GPU Duffy builder, and the list-1
evaluation with their signed arithmetic orbit reconstruction
(``volumential/orbit_arithmetic.py:176-300``: the differentiated axis fixed
and odd under reflection).  Entries are checked against the CPU Duffy
restatement and, independently of it, against central differences of the
Laplace entries in the target point; the list-1 sums against the C oracle's
signed path."""

import numpy as np
import pytest

from helpers import oracle_eval, oracle_for_workload, rel_l2
from oracle import duffy_oracle as DO
from volumential_gb300 import table_builder as TB
from volumential_gb300 import workloads as W
from volumential_gb300.kernels import (
    AxisSourceDerivative,
    AxisTargetDerivative,
    HelmholtzKernel,
    LaplaceKernel,
)
from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

pytestmark = pytest.mark.gpu


def _table(knl, q, extent):
    dt = np.complex128 if knl.is_complex_valued else np.float64
    return NearFieldInteractionTable(q, dim=knl.dim, sumpy_kernel=knl, source_box_extent=extent,
                                     dtype=dt)


@pytest.mark.parametrize("knl,kind", [
    (AxisTargetDerivative(0, LaplaceKernel(2)), "laplace"),
    (AxisSourceDerivative(1, LaplaceKernel(3)), "laplace"),
    (AxisTargetDerivative(1, HelmholtzKernel(2)), "helmholtz"),
    (AxisSourceDerivative(2, HelmholtzKernel(3)), "helmholtz")])
def test_derivative_entries_match_the_cpu_restatement(cuda, knl, kind):
    t = _table(knl, 2, 0.5)
    info = t._get_invariant_entry_info()
    assert info["kind"] == "signed-arithmetic-orbit"
    ids = info["entry_ids"]
    pick = ids[np.linspace(0, len(ids) - 1, 24 if knl.dim == 2 else 10).astype(int)]
    reg, rad = (6, 21) if knl.dim == 2 else (4, 11)
    _, got = TB.build_table_values(t, regular_quad_order=reg, radial_quad_order=rad, k=3.0,
                                   entry_ids=pick, store=False)
    tp, _, axes = TB.entry_geometry(t, pick)
    deriv = TB.kernel_derivative(knl)[1]
    ref = DO.entry_values(knl.dim, 2, 0.5, kind, tp, axes, reg, rad, k=3.0, derivative=deriv)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("dim", [2, 3])
def test_derivative_entries_are_the_gradient_of_the_laplace_entries(cuda, dim):
    # d/dt_a of the integral = the integral of d/dt_a G: central differences
    # of the Laplace entries (CPU restatement) in the target point
    knl = AxisTargetDerivative(dim - 1, LaplaceKernel(dim))
    t = _table(knl, 2, 1.0)
    ids = t._get_invariant_entry_info()["entry_ids"]
    pick = ids[np.linspace(0, len(ids) - 1, 8).astype(int)]
    reg, rad = (10, 41) if dim == 2 else (8, 31)
    _, got = TB.build_table_values(t, regular_quad_order=reg, radial_quad_order=rad,
                                   entry_ids=pick, store=False)
    tp, _, axes = TB.entry_geometry(t, pick)
    h = 1e-4
    e = np.zeros((dim, 1))
    e[dim - 1] = h
    fd = (DO.entry_values(dim, 2, 1.0, "laplace", tp + e, axes, reg, rad)
          - DO.entry_values(dim, 2, 1.0, "laplace", tp - e, axes, reg, rad)) / (2 * h)
    # O(h^2) differences: ~1e-12 relative on most entries, 2e-6 on a target
    # inside the source box (3D)
    assert np.max(np.abs(got - fd)) <= 1e-5 * np.max(np.abs(fd))


@pytest.mark.parametrize("dim,level,q", [(2, 3, 3), (3, 2, 2)])
def test_list1_with_a_derivative_table_matches_the_oracle(cuda, dim, level, q):
    torch = cuda
    knl = AxisTargetDerivative(0, LaplaceKernel(dim))
    w = W.uniform_workload("deriv", dim, level, q, seed=95, kernel=knl)
    t = _table(knl, q, w.tree.root_extent)
    t.build_table_via_duffy_radial(regular_quad_order=6, radial_quad_order=21)
    w.tables = [t]
    from helpers import wrangler_for

    wr = wrangler_for(w)
    payload = wr.get_payload(knl)
    assert payload["table_data_shapes"]["reconstruction_kind"] == "signed-arithmetic-orbit"
    tr = w.traversal
    pot, _ = wr.eval_direct(tr.target_boxes, tr.neighbor_source_boxes_starts,
                            tr.neighbor_source_boxes_lists, w.coefs[0])
    got = pot[0].cpu().numpy()
    # the inferred derivative scaling: (h / h0)^1, no displacement
    policy = {"scaling_exponent": 1, "displacement": "none", "table_level": "zero"}
    ref = oracle_eval(oracle_for_workload(w, policy), w, w.coefs[0])
    assert rel_l2(got, ref) <= 1e-12
    mixed = wr.eval_direct_batched(tr.target_boxes, tr.neighbor_source_boxes_starts,
                                   tr.neighbor_source_boxes_lists,
                                   torch.from_numpy(w.coefs[:1]).to("cuda"), precision="mixed")
    assert rel_l2(mixed[0][0].cpu().numpy(), ref) <= 1e-9
