"""Dense reconstruction (``volumential/list1.py:1018-1048``): a kernel
without the arithmetic orbit symmetry - the plane wave cos(k d_0) of the
reference's manufactured Duffy tests (``test/test_duffy_batched_manufactured.py:
219-284``) - keeps its full table (built by the FP64 GPU Duffy builder), and
the device reads it as is (``VL1_RECON_DENSE``) on the FP64 and the
tensor-core paths.  Both are checked against the numpy restatement of the
dense reads (``oracle/dense_oracle.py``) with the C oracle's case ids."""

import numpy as np
import pytest

from helpers import FIXED, rel_l2
from oracle import dense_oracle as DO
from oracle import oracle as O
from volumential_gb300.expansion_wrangler_fpnd import (
    FPNDExpansionWrangler,
    FPNDTreeIndependentDataForWrangler,
)
from volumential_gb300.kernels import PlaneWaveKernel
from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable
from volumential_gb300.tree_build import build_list1_traversal, build_uniform_tree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,level,q", [(2, 3, 3), (3, 2, 2)])
def test_dense_table_matches_the_restatement(cuda, dim, level, q):
    torch = cuda
    k = 1.7
    tree = build_uniform_tree(dim, level, q)
    trav = build_list1_traversal(tree)
    knl = PlaneWaveKernel(dim)
    t = NearFieldInteractionTable(q, dim=dim, sumpy_kernel=knl,
                                  source_box_extent=tree.root_extent * 0.5 ** level)
    t.build_table_via_duffy_radial(regular_quad_order=6, radial_quad_order=21, k=k)
    assert t.is_built and not t.table_data_is_symmetry_reduced
    assert t.data.size == t.n_cases * t.n_pairs and np.all(np.isfinite(t.data))
    ti = FPNDTreeIndependentDataForWrangler(target_kernels=[knl])
    wr = FPNDExpansionWrangler(ti, trav, [t], dtype=np.float64, quad_order=q)
    payload = wr.get_payload(knl)
    assert payload["table_data_shapes"]["reconstruction_kind"] == "dense"
    rng = np.random.default_rng(5)
    dens = rng.standard_normal((2, tree.ntargets))
    pot, _ = wr.eval_direct(trav.target_boxes, trav.neighbor_source_boxes_starts,
                            trav.neighbor_source_boxes_lists, dens[0])
    got = pot[0].cpu().numpy()
    mixed = wr.eval_direct_batched(trav.target_boxes, trav.neighbor_source_boxes_starts,
                                   trav.neighbor_source_boxes_lists,
                                   torch.from_numpy(dens).to("cuda"), precision="mixed")
    mixed = mixed[0][0].cpu().numpy()   # (per-kernel [nrhs, N] results, timing)

    info = payload["reconstruction_info"]
    md = {n: info[n] for n in ("case_orbit_ranks", "case_axis_perm", "case_axis_sign",
                               "case_axis_group", "case_value_offsets", "axis_sign_power",
                               "axis_direction_signs", "direction_sign_axis")}
    prob = O.OracleProblem(
        dim=dim, q=q, table_data=payload["table_data"], mode_nmlz=payload["mode_nmlz"],
        case_indices=payload["case_indices"], encoding_base=payload["base"],
        encoding_shift=payload["shift"], metadata=md, policy=FIXED,
        root_extent=tree.root_extent, table_root_extent=payload["table_root_extent"],
        table_starting_level=payload["table_starting_level"])
    nq = q ** dim
    full = np.asarray(payload["table_data"]).reshape(1, t.n_cases, nq, nq)
    local = tree.box_local_mode_ids()
    kw = dict(target_boxes=trav.target_boxes,
              neighbor_source_boxes_starts=trav.neighbor_source_boxes_starts,
              neighbor_source_boxes_lists=trav.neighbor_source_boxes_lists,
              box_centers=tree.box_centers, box_levels=tree.box_levels,
              box_starts=tree.box_target_starts, box_counts=tree.box_target_counts_nonchild,
              source_mode_ids=local, target_point_ids=local,
              root_extent=tree.root_extent, table_root_extent=payload["table_root_extent"])
    ref0 = DO.dense_near_field(prob, full, coefs=dens[0], **kw)
    ref1 = DO.dense_near_field(prob, full, coefs=dens[1], **kw)
    assert rel_l2(got, ref0) <= 1e-12
    assert rel_l2(mixed[0], ref0) <= 1e-9 and rel_l2(mixed[1], ref1) <= 1e-9
    # the plane wave is not invariant under swapping axes 0 and 1 (case
    # vector and both modes permuted), which the arithmetic reconstruction
    # assumes: a reduced read of the same table would be wrong
    from volumential_gb300.orbit_arithmetic import decode_mode_axes, encode_mode_axes

    def swapped_mode(m):
        ax = list(decode_mode_axes(m, q, dim))
        ax[0], ax[1] = ax[1], ax[0]
        return encode_mode_axes(ax, q)

    diffs, mags = [], []
    for c, vec in enumerate(t.interaction_case_vecs):
        v = list(vec)
        if v[0] == v[1]:
            continue
        v[0], v[1] = v[1], v[0]
        c2 = int(t.case_indices[t.case_encode(v)])
        for sm in range(nq):
            for tm in range(nq):
                a = full[0, c, sm, tm]
                b = full[0, c2, swapped_mode(sm), swapped_mode(tm)]
                diffs.append(abs(a - b))
                mags.append(abs(a))
    assert max(diffs) > 1e-3 * max(mags)
