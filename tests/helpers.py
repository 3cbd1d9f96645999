"""Helpers shared by the tests: wranglers over workloads, oracle problems."""

from __future__ import annotations

import numpy as np

from oracle import oracle as O
from volumential_gb300 import list1_gallery, orbit_arithmetic
from volumential_gb300.expansion_wrangler_fpnd import (
    FPNDExpansionWrangler,
    FPNDTreeIndependentDataForWrangler,
)

LAP2 = {"scaling_exponent": 2, "displacement": "log2d",
        "disp_coef": -0.5 / np.pi, "table_level": "zero"}
LAP3 = {"scaling_exponent": 2, "displacement": "none", "table_level": "zero"}
FIXED = {"scaling_exponent": 0, "displacement": "none", "table_level": "zero"}
PER_LEVEL = {"scaling_exponent": 0, "displacement": "none", "table_level": "per_level"}


def wrangler_for(workload, **kw):
    ti = FPNDTreeIndependentDataForWrangler(target_kernels=[workload.kernel])
    dtype = np.complex128 if workload.kernel.is_complex_valued else np.float64
    return FPNDExpansionWrangler(ti, workload.traversal, workload.tables, dtype=dtype,
                                 quad_order=workload.q, **kw)


def oracle_for_workload(workload, policy):
    """Oracle problem built from the same payload the wrangler uploads."""
    wr = wrangler_for(workload)
    payload = wr.get_payload(workload.kernel)
    info = payload["reconstruction_info"]
    md = {k: info[k] for k in ("case_orbit_ranks", "case_axis_perm", "case_axis_sign",
                               "case_axis_group", "case_value_offsets", "axis_sign_power",
                               "axis_direction_signs", "direction_sign_axis")}
    return O.OracleProblem(
        dim=workload.dim, q=workload.q, table_data=payload["table_data"],
        mode_nmlz=payload["mode_nmlz"], case_indices=payload["case_indices"],
        encoding_base=payload["base"], encoding_shift=payload["shift"], metadata=md,
        policy=policy, root_extent=workload.tree.root_extent,
        table_root_extent=payload["table_root_extent"],
        table_starting_level=payload["table_starting_level"])


def oracle_eval(problem, workload, coefs, nthreads=0):
    tr = workload.traversal
    tree = workload.tree
    local = tree.box_local_mode_ids()
    return problem.near_field(
        target_boxes=tr.target_boxes, neighbor_source_boxes_starts=tr.neighbor_source_boxes_starts,
        neighbor_source_boxes_lists=tr.neighbor_source_boxes_lists,
        box_centers=tree.box_centers, box_levels=tree.box_levels,
        box_source_starts=tree.box_target_starts,
        box_source_counts_nonchild=tree.box_target_counts_nonchild,
        box_target_starts=tree.box_target_starts,
        box_target_counts_nonchild=tree.box_target_counts_nonchild,
        source_mode_ids=local, target_point_ids=local, mode_coefs=coefs, nthreads=nthreads)


def fixture_oracle(fx):
    return O.problem_from_fixture(fx, list1_gallery, orbit_arithmetic)


def fixture_kwargs(fx):
    """NearFieldFromCSR keyword arguments of a golden list-1 fixture."""
    dim, q = int(fx["dim"]), int(fx["q"])
    prob = fixture_oracle(fx)
    vecs, _, ci = list1_gallery.generate_list1_gallery(dim)
    base, shift = list1_gallery.gallery_encoding(vecs)
    return dict(
        box_centers=fx["box_centers"], box_levels=fx["box_levels"],
        box_source_counts_nonchild=fx["box_counts"], box_source_starts=fx["box_starts"],
        box_target_counts_nonchild=fx["box_counts"], box_target_starts=fx["box_starts"],
        case_indices=ci, encoding_base=base, encoding_shift=shift,
        mode_nmlz_combined=fx["mode_nmlz"], exterior_mode_nmlz_combined=fx["mode_nmlz"],
        neighbor_source_boxes_starts=fx["starts"], root_extent=float(fx["root_extent"]),
        neighbor_source_boxes_lists=fx["lists"], mode_coefs=fx["coefs"],
        source_mode_ids=fx["source_mode_ids"], table_data_combined=fx["table_data"],
        target_boxes=fx["target_boxes"], target_point_ids=fx["target_point_ids"],
        table_root_extent=float(fx["table_root_extent"]),
        table_starting_level=int(fx["table_starting_level"]),
        arithmetic_case_orbit_ranks=prob.orbit_ranks, arithmetic_case_axis_perm=prob.perm,
        arithmetic_case_axis_sign=prob.sign, arithmetic_case_axis_group=prob.group,
        arithmetic_case_value_offsets=prob.offsets,
        arithmetic_axis_sign_power=prob.sign_power,
        arithmetic_axis_direction_signs=prob.dir_signs,
        arithmetic_direction_sign_axis=int(prob.params.direction_sign_axis)), prob


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


MIXED_TREE_KEYS = ("target_boxes", "neighbor_source_boxes_starts",
                   "neighbor_source_boxes_lists", "box_centers", "box_levels",
                   "box_source_starts", "box_source_counts_nonchild", "box_target_starts",
                   "box_target_counts_nonchild", "source_mode_ids", "target_point_ids")


def plan_and_view(w):
    """(plan, tree view, kept device arrays) of a workload, for calls that go
    below the wrangler (schedules, C ABI entry points)."""
    from volumential_gb300.plan import tree_view_from_arrays

    wr = wrangler_for(w)
    tr = w.traversal
    payload = wr.get_payload(w.kernel)
    nf = wr.near_field_evaluator(w.kernel, payload)
    kw = wr._near_field_kwargs(payload, tr.target_boxes, tr.neighbor_source_boxes_starts,
                               tr.neighbor_source_boxes_lists, None)
    plan = nf.get_plan(
        table_data_combined=kw["table_data_combined"],
        mode_nmlz_combined=kw["mode_nmlz_combined"], case_indices=kw["case_indices"],
        encoding_base=kw["encoding_base"], encoding_shift=kw["encoding_shift"],
        table_root_extent=kw["table_root_extent"],
        table_starting_level=kw["table_starting_level"],
        **{n: kw[n] for n in kw if n.startswith("arithmetic_")})
    view, keep = tree_view_from_arrays(root_extent=kw["root_extent"],
                                       **{k: kw[k] for k in MIXED_TREE_KEYS})
    return plan, view, keep
