"""The oracle and the host-side index code against the reference's golden vectors.

Fixtures in ``tests/golden`` were produced from the reference by
``tests/golden/make_golden.py`` (gallery, orbit metadata, full index-map
digests, end-to-end list-1 results of a line-by-line restatement of
``volumential/list1.py:1060-1139`` using the reference's own orbit index).
"""

import glob
import hashlib
import os

import numpy as np
import pytest

from helpers import fixture_oracle, rel_l2
from oracle import oracle as O
from volumential_gb300 import list1_gallery as gal
from volumential_gb300 import orbit_arithmetic as oa
from volumential_gb300.expansion_wrangler_fpnd import (
    _build_fast_scalar_arithmetic_orbit_reconstruction,
    _prepare_table_data_and_entry_map,
)
from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ORBIT_FILES = sorted(glob.glob(os.path.join(GOLDEN, "orbit_*.npz")))
LIST1_FILES = sorted(glob.glob(os.path.join(GOLDEN, "list1_*.npz")))


class _TableLike:
    def __init__(self, dim, q):
        self.dim, self.quad_order = dim, q
        self.interaction_case_vecs, self.case_encode, self.case_indices = \
            gal.generate_list1_gallery(dim)
        self.n_cases = len(self.interaction_case_vecs)
        self.n_q_points = q ** dim
        self.n_pairs = q ** (2 * dim)


def _signed_symmetry(dim):
    return {"axis_groups": ((0,), tuple(range(1, dim))),
            "axis_sign_power": np.array([1] + [0] * (dim - 1), dtype=np.uint8),
            "axis_direction_signs": np.zeros(dim, dtype=np.int8),
            "direction_sign_axis": -1}


def _parse_orbit_name(path):
    name = os.path.basename(path)
    dim = int(name.split("_d")[1][0])
    q = int(name.split("_q")[1].split(".")[0])
    return name, dim, q, "signed" in name


# {{{ gallery (test/test_list1_gallery.py:27-64)

def test_gallery_matches_reference():
    g = np.load(os.path.join(GOLDEN, "gallery.npz"))
    for dim in (2, 3):
        vecs, enc, ci = gal.generate_list1_gallery(dim)
        assert np.array_equal(np.asarray(vecs), g[f"vecs{dim}"])
        assert np.array_equal(ci, g[f"case_indices{dim}"])
        for cid, v in enumerate(vecs):
            assert ci[enc(v)] == cid


def test_gallery_counts():
    v1, _, _ = gal.generate_list1_gallery(1)
    assert len(v1) == 7
    v2, _, _ = gal.generate_list1_gallery(2)
    assert len(v2) == 8 + 12 + 12 + 1
    nums = {c for v in v2 for c in v}
    assert len(nums) == 11 and max(nums) == 6 and min(nums) == -6
    v3, _, ci3 = gal.generate_list1_gallery(3)
    assert len(v3) == 139 and ci3.size == 13 ** 3
    assert gal.gallery_encoding(v3) == (13, 6)

# }}}


# {{{ orbit metadata, representatives, full maps

@pytest.mark.parametrize("path", ORBIT_FILES, ids=[os.path.basename(p) for p in ORBIT_FILES])
def test_orbit_metadata_matches_reference(path):
    name, dim, q, signed = _parse_orbit_name(path)
    fx = np.load(path)
    md = oa.build_arithmetic_case_metadata(_TableLike(dim, q),
                                           _signed_symmetry(dim) if signed else None)
    for key in ("canonical_case_ids", "case_orbit_ranks", "case_axis_perm",
                "case_axis_sign", "case_axis_group", "case_value_offsets",
                "axis_sign_power", "axis_direction_signs"):
        assert np.array_equal(md[key], fx[key]), key
    assert md["n_compact_entries"] == int(fx["n_compact_entries"])
    reps = oa.enumerate_scalar_arithmetic_representatives(_TableLike(dim, q), md)
    assert np.array_equal(reps, fx["representatives"])


@pytest.mark.parametrize("path", ORBIT_FILES, ids=[os.path.basename(p) for p in ORBIT_FILES])
def test_oracle_full_index_map_digest(path):
    """Every (case, source mode, target point) row and sign, bit-exact."""
    name, dim, q, signed = _parse_orbit_name(path)
    fx = np.load(path)
    t = _TableLike(dim, q)
    md = oa.build_arithmetic_case_metadata(t, _signed_symmetry(dim) if signed else None)
    base, shift = gal.gallery_encoding(t.interaction_case_vecs)
    prob = O.OracleProblem(dim=dim, q=q, table_data=np.zeros((1, md["n_compact_entries"])),
                           mode_nmlz=np.zeros((1, q ** dim)), case_indices=t.case_indices,
                           encoding_base=base, encoding_shift=shift, metadata=md,
                           policy={"scaling_exponent": 0}, root_extent=1.0,
                           table_root_extent=1.0)
    rows, signs = prob.full_map()
    h = hashlib.sha256()
    h.update(rows.astype("<i4").tobytes())
    h.update(signs.astype("i1").tobytes())
    assert h.hexdigest() == str(fx["map_sha256"])
    c, s, tt = fx["sample_case"], fx["sample_src"], fx["sample_tgt"]
    assert np.array_equal(rows[c, s, tt], fx["sample_row"])
    assert np.array_equal(signs[c, s, tt], fx["sample_sign"])


@pytest.mark.parametrize("path", ORBIT_FILES[:6], ids=[os.path.basename(p) for p in ORBIT_FILES[:6]])
def test_python_entry_evaluator_samples(path):
    name, dim, q, signed = _parse_orbit_name(path)
    fx = np.load(path)
    md = oa.build_arithmetic_case_metadata(_TableLike(dim, q),
                                           _signed_symmetry(dim) if signed else None)
    for c, s, t, r, sg in list(zip(fx["sample_case"], fx["sample_src"], fx["sample_tgt"],
                                   fx["sample_row"], fx["sample_sign"]))[:500]:
        assert oa.evaluate_compact_arithmetic_entry(int(c), int(s), int(t), md, q, dim) \
            == (int(r), int(sg))


def test_representatives_map_to_their_own_rows():
    """Every enumerated representative reconstructs to its own compact row."""
    for dim, q in ((2, 4), (3, 3)):
        t = _TableLike(dim, q)
        md = oa.build_arithmetic_case_metadata(t)
        reps = oa.enumerate_scalar_arithmetic_representatives(t, md)
        nq = q ** dim
        for row, e in enumerate(reps.tolist()):
            c, rem = divmod(e, nq * nq)
            s, tt = divmod(rem, nq)
            assert oa.evaluate_compact_arithmetic_entry(c, s, tt, md, q, dim)[0] == row

# }}}


# {{{ reference known-answer tests

def test_sorting_network_sorts_nonadjacent_group_axes():
    """test/test_nearfield_potential_table.py:2361-2384 (q=3, groups [1,0,1])."""
    q = 3
    md = {"case_orbit_ranks": np.array([0], dtype=np.uint16),
          "case_value_offsets": np.array([0, 10 ** 6], dtype=np.int32),
          "case_axis_perm": np.array([[0, 1, 2]], dtype=np.uint8),
          "case_axis_sign": np.array([[1, 1, 1]], dtype=np.int8),
          "case_axis_group": np.array([[1, 0, 1]], dtype=np.uint8),
          "axis_sign_power": np.zeros(3, dtype=np.uint8),
          "axis_direction_signs": np.zeros(3, dtype=np.int8),
          "direction_sign_axis": -1}
    s = t = 2 * q * q
    # the oracle (generated-kernel formulation) must sort axes 0 and 2
    prob = O.OracleProblem(dim=3, q=q, table_data=np.zeros((1, 10 ** 6)),
                           mode_nmlz=np.zeros((1, 27)), case_indices=np.zeros(2197),
                           encoding_base=13, encoding_shift=6, metadata=md,
                           policy={"scaling_exponent": 0}, root_extent=1.0,
                           table_root_extent=1.0)
    prob.params.n_cases = 1
    rows, signs = prob.full_map()
    row_py, sign_py = oa.evaluate_compact_arithmetic_entry(0, s, t, md, q, 3)
    assert rows[0, s, t] == row_py and signs[0, s, t] == sign_py == 1
    # the reference's known answer: canonical mode 2 for source and target
    full, sign = oa.evaluate_arithmetic_orbit_entry(0, s, t, md, q, 3)
    assert full == 2 * 27 + 2 and sign == 1


def test_q3_3d_payload_diagnostic_counts():
    """test/test_nearfield_potential_table.py:2633-2671."""
    t = NearFieldInteractionTable(3, dim=3)
    info = t._get_scalar_arithmetic_invariant_entry_info()
    ids = info["entry_ids"]
    t.set_reduced_table_data(ids, np.arange(1, len(ids) + 1, dtype=np.float64))
    tdc, _, _, entry_ids, entry_scales, recon = _prepare_table_data_and_entry_map([t])
    assert recon["kind"] == "scalar-arithmetic-orbit"
    assert tdc.shape[1] == len(ids) == 2510
    assert recon["compact_value_entry_count"] == 2510
    assert recon["representative_entry_count"] == 2510
    assert recon["dense_arithmetic_layout_entry_count"] == 7290
    assert recon["unused_layout_entry_count"] == 0
    assert entry_ids.nbytes + entry_scales.nbytes == 0
    assert recon["metadata_bytes"] == 1576
    assert np.array_equal(tdc[0], np.arange(1, 2511, dtype=np.float64))


@pytest.mark.parametrize("q", [1, 2, 3, 5, 8])
def test_normalizers_are_gauss_legendre_weight_products(q):
    """test/test_nearfield_potential_table.py:310-330."""
    t = NearFieldInteractionTable(q, dim=2)
    t.build_normalizer_table()
    _, w = np.polynomial.legendre.leggauss(q)
    w = 0.5 * t.source_box_extent * w
    assert np.allclose(t.mode_normalizers, np.multiply.outer(w, w).reshape(-1),
                       rtol=0, atol=256 * np.finfo(np.float64).eps)


def test_compact_counts_of_the_configs():
    for dim, q, n in ((2, 4, 1084), (2, 5, 2641), (3, 3, 2510), (3, 4, 12936),
                      (3, 5, 48230)):
        md = oa.build_arithmetic_case_metadata(_TableLike(dim, q))
        assert md["n_compact_entries"] == n
        assert len(md["canonical_case_ids"]) == (7 if dim == 2 else 10)

# }}}


# {{{ end-to-end list-1 goldens

@pytest.mark.parametrize("path", LIST1_FILES, ids=[os.path.basename(p) for p in LIST1_FILES])
def test_oracle_reproduces_reference_list1_bit_exactly(path):
    fx = np.load(path)
    prob = fixture_oracle(fx)
    res = prob.near_field(
        target_boxes=fx["target_boxes"], neighbor_source_boxes_starts=fx["starts"],
        neighbor_source_boxes_lists=fx["lists"], box_centers=fx["box_centers"],
        box_levels=fx["box_levels"], box_source_starts=fx["box_starts"],
        box_source_counts_nonchild=fx["box_counts"], box_target_starts=fx["box_starts"],
        box_target_counts_nonchild=fx["box_counts"], source_mode_ids=fx["source_mode_ids"],
        target_point_ids=fx["target_point_ids"], mode_coefs=fx["coefs"])
    assert np.array_equal(res, fx["result"])


@pytest.mark.parametrize("name", ["constant2d_q1", "constant2d_q2", "constant3d_q1",
                                  "constant3d_q2"])
def test_completeness_constant_kernel(name):
    """test/test_nearfield_interaction_completeness.py:44-207: density 1 and a
    constant-kernel table give 2**dim at every target."""
    fx = np.load(os.path.join(GOLDEN, f"list1_{name}.npz"))
    dim = int(fx["dim"])
    assert np.all(np.abs(fx["result"] - 2 ** dim) < 1e-8)


def test_oracle_reports_invalid_case():
    """A pair whose case code is outside the gallery is reported, not read."""
    fx = np.load(os.path.join(GOLDEN, "list1_lap2d_uniform_l3_q3.npz"))
    prob = fixture_oracle(fx)
    centers = fx["box_centers"].copy()
    t0 = int(fx["target_boxes"][0])
    centers[0, t0] += 0.37 * (centers[0, 1] - centers[0, 0] + 1.0)
    res, status = prob.near_field(
        target_boxes=fx["target_boxes"], neighbor_source_boxes_starts=fx["starts"],
        neighbor_source_boxes_lists=fx["lists"], box_centers=centers,
        box_levels=fx["box_levels"], box_source_starts=fx["box_starts"],
        box_source_counts_nonchild=fx["box_counts"], box_target_starts=fx["box_starts"],
        box_target_counts_nonchild=fx["box_counts"], source_mode_ids=fx["source_mode_ids"],
        target_point_ids=fx["target_point_ids"], mode_coefs=fx["coefs"], check=False)
    assert status == 1

# }}}


def test_fast_reconstruction_info_shape():
    t = NearFieldInteractionTable(4, dim=2)
    t.build_constant_table()
    info = _build_fast_scalar_arithmetic_orbit_reconstruction(t)
    assert info["kind"] == "scalar-arithmetic-orbit"
    assert info["n_case_orbits"] == 7
    assert info["compact_value_entry_count"] == 1084
    assert rel_l2(t.get_entry_data_for_full_indices(info["layout_entry_ids"]),
                  t.mode_weights()[info["layout_entry_ids"] % 256 // 16]) == 0.0


@pytest.mark.parametrize("dim", [2, 3])
def test_derivative_kernel_tables_take_the_reference_signed_descriptors(dim):
    # the symmetry derived from AxisTargetDerivative(0, Laplace) (orbit_arithmetic.py:
    # 176-300) gives the signed descriptors and representatives that the
    # reference's own module produced for that kernel
    from volumential_gb300.kernels import AxisTargetDerivative, LaplaceKernel
    from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

    fx = np.load(os.path.join(GOLDEN, f"orbit_signed_d{dim}_q3.npz"))
    knl = AxisTargetDerivative(0, LaplaceKernel(dim))
    t = NearFieldInteractionTable(3, dim=dim, sumpy_kernel=knl)
    info = t._get_invariant_entry_info()
    assert info["kind"] == "signed-arithmetic-orbit"
    md = info["arithmetic_metadata"]
    for key in ("case_orbit_ranks", "case_axis_perm", "case_axis_sign", "case_axis_group",
                "case_value_offsets", "axis_sign_power", "axis_direction_signs"):
        assert np.array_equal(np.asarray(md[key]), fx[key]), key
    assert np.array_equal(info["entry_ids"], fx["representatives"])
