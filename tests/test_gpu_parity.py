"""GPU parity of the plain FP64 list-1 path (through the C ABI).

* the device-computed orbit index map is bit-exact against the reference's
  full-map digests and against the oracle;
* every end-to-end golden of the reference is reproduced within 1e-12
  relative l2 (plain FP64 path tolerance);
* larger seeded workloads (config-1 shape, adaptive 2D/3D, complex tables,
  many right-hand sides) match the C oracle within 1e-12;
* invalid inputs raise host exceptions, without faulting the device.
"""

import glob
import hashlib
import os

import numpy as np
import pytest

from helpers import (
    FIXED,
    LAP2,
    LAP3,
    fixture_kwargs,
    oracle_eval,
    oracle_for_workload,
    rel_l2,
    wrangler_for,
)
from volumential_gb300 import list1_gallery as gal
from volumential_gb300 import orbit_arithmetic as oa
from volumential_gb300.kernels import AxisTargetDerivative, HelmholtzKernel, LaplaceKernel
from volumential_gb300.list1 import NearFieldFromCSR
from volumential_gb300.plan import Plan
from volumential_gb300.volume_fmm import drive_volume_fmm
from volumential_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ORBIT_FILES = sorted(glob.glob(os.path.join(GOLDEN, "orbit_*.npz")))
LIST1_FILES = sorted(glob.glob(os.path.join(GOLDEN, "list1_*.npz")))
TOL_FP64 = 1e-12


def _kernel_for_fixture(name, dim):
    if name.startswith("helm2d"):
        return HelmholtzKernel(2), {}
    if name.startswith("perlevel"):
        return LaplaceKernel(dim), {"infer_kernel_scaling": False}
    if name.startswith("signed"):
        return AxisTargetDerivative(0, LaplaceKernel(dim)), {}
    return LaplaceKernel(dim), {}


@pytest.mark.parametrize("path", ORBIT_FILES, ids=[os.path.basename(p) for p in ORBIT_FILES])
def test_device_orbit_index_map_is_bit_exact(path, cuda):
    name = os.path.basename(path)
    dim = int(name.split("_d")[1][0])
    q = int(name.split("_q")[1].split(".")[0])
    fx = np.load(path)
    vecs, _, ci = gal.generate_list1_gallery(dim)
    base, shift = gal.gallery_encoding(vecs)
    n = int(fx["n_compact_entries"])
    plan = Plan(dim=dim, quad_order=q, n_tables=1, table_data=np.zeros((1, n)),
                mode_nmlz=np.zeros((1, q ** dim)), case_indices=ci, encoding_base=base,
                encoding_shift=shift, case_encoding_bias=1e-10,
                case_orbit_ranks=fx["case_orbit_ranks"], case_axis_perm=fx["case_axis_perm"],
                case_axis_sign=fx["case_axis_sign"], case_axis_group=fx["case_axis_group"],
                case_value_offsets=fx["case_value_offsets"],
                axis_sign_power=fx["axis_sign_power"],
                axis_direction_signs=fx["axis_direction_signs"],
                direction_sign_axis=int(fx["direction_sign_axis"]),
                reconstruction_kind=1 if "signed" in name else 0, scaling_exponent=0,
                displacement_kind=0, displacement_coef=0.0, table_level_kind=0,
                table_root_extent=1.0, table_starting_level=0)
    rows, signs = plan.orbit_index_map()
    rows = rows.cpu().numpy()
    signs = signs.cpu().numpy()
    h = hashlib.sha256()
    h.update(rows.astype("<i4").tobytes())
    h.update(signs.astype("i1").tobytes())
    assert h.hexdigest() == str(fx["map_sha256"])
    plan.destroy()


@pytest.mark.parametrize("path", LIST1_FILES, ids=[os.path.basename(p) for p in LIST1_FILES])
def test_golden_list1_through_near_field_from_csr(path, cuda):
    fx = np.load(path)
    name = os.path.basename(path)[len("list1_"):-4]
    dim = int(fx["dim"])
    kw, prob = fixture_kwargs(fx)
    knl, extra = _kernel_for_fixture(name, dim)
    shapes = {"n_tables": int(fx["n_tables"]), "quad_order": int(fx["q"]),
              "n_q_points": int(fx["q"]) ** dim, "n_cases": len(gal.generate_list1_gallery(dim)[0]),
              "n_table_entries": int(fx["table_data"].shape[1]),
              "reconstruction_kind": "signed-arithmetic-orbit" if name.startswith("signed")
              else "scalar-arithmetic-orbit",
              "n_arithmetic_case_orbits": int(prob.offsets.size - 1)}
    nf = NearFieldFromCSR(knl, shapes, **extra)
    out_dtype = cuda.complex128 if np.iscomplexobj(fx["result"]) else cuda.float64
    result = cuda.zeros(len(fx["result"]), dtype=out_dtype, device="cuda")
    res, evt = nf(None, result=result, **kw)
    assert res is result
    got = res.cpu().numpy()
    assert rel_l2(got, fx["result"]) <= TOL_FP64
    if name.startswith("constant"):
        assert np.max(np.abs(got - 2 ** dim)) < 1e-12


def _check_workload(w, policy, tol=TOL_FP64):
    wr = wrangler_for(w)
    prob = oracle_for_workload(w, policy)
    tr = w.traversal
    pots, _ = wr.eval_direct(tr.target_boxes, tr.neighbor_source_boxes_starts,
                             tr.neighbor_source_boxes_lists, w.coefs[0])
    got = pots[0].cpu().numpy()
    ref = oracle_eval(prob, w, w.coefs[0])
    err = rel_l2(got, ref)
    assert err <= tol, err
    return wr, prob


def test_config1_shape_2d_laplace_uniform_l5_q4(cuda):
    _check_workload(W.config_c1(seed=11), LAP2)


def test_2d_laplace_adaptive_q3(cuda):
    w = W.adaptive_workload("a2", 2, 3, tol=1e-3, max_level=7, min_level=2, seed=12,
                            n_terms=8, width_range=(0.02, 0.1))
    assert len(np.unique(w.tree.box_levels[w.traversal.target_boxes])) > 1
    _check_workload(w, LAP2)


def test_3d_laplace_adaptive_q4(cuda):
    w = W.adaptive_workload("a3", 3, 4, tol=3e-2, max_level=5, min_level=2, seed=13)
    assert len(np.unique(w.tree.box_levels[w.traversal.target_boxes])) > 1
    _check_workload(w, LAP3)


def test_3d_laplace_uniform_q5(cuda):
    _check_workload(W.uniform_workload("u3", 3, 2, 5, seed=14), LAP3)


def test_2d_helmholtz_complex_fixed_table(cuda):
    w = W.uniform_workload("h2", 2, 4, 4, seed=15, kernel=HelmholtzKernel(2),
                           complex_table=True)
    w.tables = W.synthetic_tables(2, 4, w.kernel, seed=5, complex_values=True,
                                  source_box_extent=w.tree.root_extent / 16)
    _check_workload(w, FIXED)


def test_many_rhs_batched_fp64_matches_per_rhs_oracle(cuda):
    w = W.uniform_workload("m", 2, 4, 4, seed=16, nrhs=5)
    wr = wrangler_for(w)
    prob = oracle_for_workload(w, LAP2)
    tr = w.traversal
    outs, _ = wr.eval_direct_batched(tr.target_boxes, tr.neighbor_source_boxes_starts,
                                     tr.neighbor_source_boxes_lists, w.coefs)
    got = outs[0].cpu().numpy()
    for r in range(w.nrhs):
        assert rel_l2(got[r], oracle_eval(prob, w, w.coefs[r])) <= TOL_FP64


def test_drive_volume_fmm_list1_superposes_fields(cuda):
    w = W.uniform_workload("d", 3, 2, 3, seed=17, nrhs=3)
    wr = wrangler_for(w)
    prob = oracle_for_workload(w, LAP3)
    sf = np.empty(3, dtype=object)
    sf[:] = [w.coefs[i] for i in range(3)]
    res = drive_volume_fmm(w.traversal, wr, sf, sf, list1_only=True)
    ref = sum(oracle_eval(prob, w, w.coefs[i]) for i in range(3))
    assert rel_l2(res[0].cpu().numpy(), ref) <= TOL_FP64
    single = drive_volume_fmm(w.traversal, wr, w.coefs[0], w.coefs[0], list1_only=True)
    assert rel_l2(single[0].cpu().numpy(), oracle_eval(prob, w, w.coefs[0])) <= TOL_FP64


def test_complex_coefficients_with_real_table(cuda):
    w = W.uniform_workload("cc", 2, 3, 3, seed=18)
    coefs = w.coefs[0] + 1j * np.roll(w.coefs[0], 7)
    wr = wrangler_for(w)
    prob = oracle_for_workload(w, LAP2)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, coefs)
    out = cuda.zeros(w.n_points, dtype=cuda.complex128, device="cuda")
    res, _ = nf(None, result=out, **kw)
    assert rel_l2(res.cpu().numpy(), oracle_eval(prob, w, coefs)) <= TOL_FP64


def test_side_stream_and_numpy_result(cuda):
    w = W.uniform_workload("s", 2, 3, 4, seed=19)
    wr = wrangler_for(w)
    prob = oracle_for_workload(w, LAP2)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, w.coefs[0])
    s = cuda.cuda.Stream()
    host = np.zeros(w.n_points)
    res, evt = nf(s, result=host, **kw)
    evt.synchronize()
    assert res is host
    assert rel_l2(host, oracle_eval(prob, w, w.coefs[0])) <= TOL_FP64


def test_invalid_case_raises_and_device_stays_usable(cuda):
    w = W.uniform_workload("bad", 2, 3, 3, seed=20)
    wr = wrangler_for(w)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, w.coefs[0])
    kw["box_centers"] = kw["box_centers"].copy()
    kw["box_centers"][0, tr.target_boxes[5]] += 0.3 / 8
    out = cuda.zeros(w.n_points, dtype=cuda.float64, device="cuda")
    with pytest.raises(RuntimeError, match="outside the interaction gallery"):
        nf(None, result=out, **kw)
    # a valid call on the same plan still works
    _check_workload(w, LAP2)


def test_layout_violation_raises(cuda):
    w = W.uniform_workload("lay", 2, 3, 3, seed=21)
    wr = wrangler_for(w)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, w.coefs[0])
    good_modes = kw["source_mode_ids"].copy()
    modes = good_modes.copy()
    modes[3] = 99
    kw["source_mode_ids"] = modes
    out = cuda.zeros(w.n_points, dtype=cuda.float64, device="cuda")
    with pytest.raises(ValueError, match="quadrature points per active"):
        nf(None, result=out, **kw)
    kw["source_mode_ids"] = good_modes
    bad_lists = np.array(tr.neighbor_source_boxes_lists).copy()
    bad_lists[0] = w.tree.nboxes + 5
    kw["neighbor_source_boxes_lists"] = bad_lists
    with pytest.raises(ValueError, match="invalid list-1 tree arrays"):
        nf(None, result=out, **kw)


def test_single_table_level_mismatch_raises(cuda):
    w = W.uniform_workload("lvl", 2, 3, 3, seed=22, kernel=HelmholtzKernel(2),
                           complex_table=True)
    w.tables = W.synthetic_tables(2, 3, w.kernel, seed=5, complex_values=True,
                                  source_box_extent=w.tree.root_extent / 4)
    wr = wrangler_for(w)
    tr = w.traversal
    with pytest.raises(RuntimeError, match="level mismatch"):
        wr.eval_direct(tr.target_boxes, tr.neighbor_source_boxes_starts,
                       tr.neighbor_source_boxes_lists, w.coefs[0])
