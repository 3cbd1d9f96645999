"""Generate the golden fixtures of the list-1 path from the reference itself.

Run in a container where the reference source tree is mounted (read only):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/reference

Only the reference modules that depend on numpy alone are imported (by file
path, without importing the ``volumential`` package, whose ``__init__`` needs
pytools): ``volumential/list1_gallery.py`` and ``volumential/orbit_arithmetic.py``.
They give the exact case encoding and the exact integer orbit index of the
reference.  The list-1 main loop itself (``volumential/list1.py:1060-1139``)
is generated OpenCL in the reference and needs loopy/pyopencl, so this script
restates that loop line by line in plain Python, calling the reference's own
``_evaluate_compact_arithmetic_orbit_entry`` for every table row.

Outputs (all small, committed):

* ``gallery.npz``        case vectors, base, shift and case_indices, 2D and 3D
* ``orbit_d{d}_q{q}.npz`` case metadata, representative entry ids, SHA-256 of
                          the full (row, sign) map over all cases x modes x
                          points, and a seeded sample of explicit entries
* ``orbit_signed_*.npz``  the same for derivative-kernel (signed) descriptors
* ``list1_*.npz``         end-to-end list-1 inputs and the restated result
"""

from __future__ import annotations

import hashlib
import importlib.util
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.dont_write_bytecode = True


def load_ref(ref_root, name):
    path = os.path.join(ref_root, "volumential", f"{name}.py")
    spec = importlib.util.spec_from_file_location(f"_ref_{name}", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class TableLike:
    def __init__(self, gal, dim, q):
        vecs, enc, ci = gal.generate_list1_gallery(dim)
        self.dim = dim
        self.quad_order = q
        self.interaction_case_vecs = vecs
        self.case_encode = enc
        self.case_indices = ci
        self.n_cases = len(vecs)
        self.n_q_points = q ** dim
        self.n_pairs = q ** (2 * dim)


def full_map(oa, md, q, dim, n_cases):
    nq = q ** dim
    rows = np.empty((n_cases, nq, nq), dtype=np.int32)
    signs = np.empty((n_cases, nq, nq), dtype=np.int8)
    for c in range(n_cases):
        for s in range(nq):
            for t in range(nq):
                r, sg = oa._evaluate_compact_arithmetic_orbit_entry(
                    c, s, t,
                    case_orbit_ranks=md["case_orbit_ranks"],
                    case_value_offsets=md["case_value_offsets"],
                    case_axis_perm=md["case_axis_perm"],
                    case_axis_sign=md["case_axis_sign"],
                    case_axis_group=md["case_axis_group"],
                    axis_sign_power=md["axis_sign_power"],
                    axis_direction_signs=md["axis_direction_signs"],
                    direction_sign_axis=md["direction_sign_axis"],
                    q_order=q, dim=dim)
                rows[c, s, t] = r
                signs[c, s, t] = sg
    return rows, signs


def digest(rows, signs):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rows, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(signs, dtype="i1").tobytes())
    return h.hexdigest()


def save_orbit(path, md, reps, rows, signs, seed):
    rng = np.random.default_rng(seed)
    n_cases, nq, _ = rows.shape
    k = min(4000, rows.size)
    flat = rng.choice(rows.size, size=k, replace=False)
    c, rem = np.divmod(flat, nq * nq)
    s, t = np.divmod(rem, nq)
    np.savez_compressed(
        path,
        canonical_case_ids=md["canonical_case_ids"],
        case_orbit_ranks=md["case_orbit_ranks"],
        case_axis_perm=md["case_axis_perm"],
        case_axis_sign=md["case_axis_sign"],
        case_axis_group=md["case_axis_group"],
        case_value_offsets=md["case_value_offsets"],
        axis_sign_power=md["axis_sign_power"],
        axis_direction_signs=md["axis_direction_signs"],
        direction_sign_axis=np.int64(md["direction_sign_axis"]),
        n_compact_entries=np.int64(md["n_compact_entries"]),
        representatives=reps,
        map_sha256=np.array(digest(rows, signs)),
        sample_case=c.astype(np.int32), sample_src=s.astype(np.int32),
        sample_tgt=t.astype(np.int32),
        sample_row=rows[c, s, t], sample_sign=signs[c, s, t])


# {{{ small trees (explicit, independent of the package's builder)

def uniform_tree(dim, level, q, a, b):
    import itertools
    boxes = []
    for lev in range(level + 1):
        n = 1 << lev
        for idx in itertools.product(range(n), repeat=dim):
            boxes.append((lev, idx))
    return tree_from_boxes(boxes, dim, q, a, b)


def adaptive_tree_2d(q, a, b):
    """A hand-made 2:1 balanced quadtree with leaves on levels 2..4."""
    import itertools
    leaves = set()
    for idx in itertools.product(range(4), repeat=2):
        leaves.add((2, idx))
    # refine (1,1) at level 2 and one of its children again
    def refine(box):
        lev, (i, j) = box
        leaves.remove(box)
        for di, dj in itertools.product((0, 1), repeat=2):
            leaves.add((lev + 1, (2 * i + di, 2 * j + dj)))
    refine((2, (1, 1)))
    refine((3, (3, 3)))
    # balance: level-4 boxes at (6..7, 6..7) touch level-2 boxes (2,*) -> refine those
    for box in [(2, (2, 1)), (2, (1, 2)), (2, (2, 2))]:
        refine(box)
    return tree_from_leaves(sorted(leaves), 2, q, a, b)


def adaptive_tree_3d(q, a, b):
    import itertools
    leaves = set()
    for idx in itertools.product(range(2), repeat=3):
        leaves.add((1, idx))
    lev, idx = 1, (0, 0, 0)
    leaves.remove((lev, idx))
    for d in itertools.product((0, 1), repeat=3):
        leaves.add((2, d))
    return tree_from_leaves(sorted(leaves), 3, q, a, b)


def tree_from_leaves(leaves, dim, q, a, b):
    boxes = set()
    for lev, idx in leaves:
        cur = (lev, tuple(idx))
        while True:
            boxes.add(cur)
            if cur[0] == 0:
                break
            cur = (cur[0] - 1, tuple(i // 2 for i in cur[1]))
    return tree_from_boxes(sorted(boxes), dim, q, a, b, leaves=set(
        (lev, tuple(idx)) for lev, idx in leaves))


def tree_from_boxes(boxes, dim, q, a, b, leaves=None):
    boxes = sorted(boxes)
    if leaves is None:
        maxlev = max(lev for lev, _ in boxes)
        leaves = {bx for bx in boxes if bx[0] == maxlev}
    nb = len(boxes)
    nb_al = ((nb + 31) // 32) * 32
    extent = b - a
    centers = np.zeros((dim, nb_al))
    levels = np.zeros(nb, dtype=np.uint8)
    for i, (lev, idx) in enumerate(boxes):
        h = extent / 2 ** lev
        centers[:, i] = [a + (k + 0.5) * h for k in idx]
        levels[i] = lev
    leaf_ids = [i for i, bx in enumerate(boxes) if bx in leaves]
    nq = q ** dim
    starts = np.zeros(nb, dtype=np.int32)
    counts = np.zeros(nb, dtype=np.int32)
    for k, i in enumerate(leaf_ids):
        starts[i] = k * nq
        counts[i] = nq
    # list 1: touching leaves (closure intersection), self included
    lists, st = [], [0]
    for t in leaf_ids:
        ht = extent / 2 ** int(levels[t])
        row = []
        for s in leaf_ids:
            hs = extent / 2 ** int(levels[s])
            gap = np.max(np.abs(centers[:, t] - centers[:, s]) - 0.5 * (ht + hs))
            if gap <= 1e-12 * extent:
                row.append(s)
        lists.extend(row)
        st.append(len(lists))
    return dict(box_centers=centers, box_levels=levels, box_starts=starts,
                box_counts=counts, target_boxes=np.array(leaf_ids, dtype=np.int32),
                starts=np.array(st, dtype=np.int32), lists=np.array(lists, dtype=np.int32),
                root_extent=float(extent), n_points=len(leaf_ids) * nq)

# }}}


def restated_near_field(inp, md, oa, q, dim, n_tables, table_data, mode_nmlz,
                        case_indices, base, shift, bias, policy, table_root_extent,
                        table_starting_level, coefs, smode, tmode):
    """``volumential/list1.py:1060-1139`` restated literally (potential_kind=1)."""
    n_tables_ = n_tables
    result = np.zeros(inp["n_points"], dtype=np.result_type(table_data.dtype, coefs.dtype))
    cache = {}
    centers = inp["box_centers"]
    root_extent = inp["root_extent"]
    for tbox, tid_box in enumerate(inp["target_boxes"]):
        tbeg = inp["box_starts"][tid_box]
        ntgt = inp["box_counts"][tid_box]
        for tid in range(q ** dim):
            if tid >= ntgt:
                continue
            target_id = tbeg + tid
            acc = 0.0
            for isb in range(inp["starts"][tbox], inp["starts"][tbox + 1]):
                sbox = inp["lists"][isb]
                nsrc = inp["box_counts"][sbox]
                sbeg = inp["box_starts"][sbox]
                slev = int(inp["box_levels"][sbox])
                sbox_extent = root_extent * (1.0 / (2 ** slev))
                if policy["table_level"] == "zero":
                    table_lev = 0
                else:
                    d = slev - table_starting_level
                    table_lev = 0 if slev < table_starting_level else (
                        d if d < n_tables_ else n_tables_ - 1)
                v = 0.0
                for ax in range(dim):
                    comp = ((centers[ax, tid_box] - centers[ax, sbox]) / sbox_extent * 4.0
                            + shift + bias)
                    v = v * base + comp
                vec_id = int(v + 0.5)
                case_id = int(case_indices[vec_id])
                assert case_id >= 0, "tree is not 2:1 balanced"
                p = policy["scaling_exponent"]
                if p == 0:
                    scaling = 1.0
                else:
                    num = sbox_extent
                    den = table_root_extent
                    for _ in range(abs(p) - 1):
                        num = num * sbox_extent
                        den = den * table_root_extent
                    scaling = num / den if p > 0 else den / num
                for sid in range(nsrc):
                    source_id = sbeg + sid
                    sm = int(smode[source_id])
                    tp = int(tmode[target_id])
                    key = (case_id, sm, tp)
                    if key not in cache:
                        cache[key] = oa._evaluate_compact_arithmetic_orbit_entry(
                            case_id, sm, tp,
                            case_orbit_ranks=md["case_orbit_ranks"],
                            case_value_offsets=md["case_value_offsets"],
                            case_axis_perm=md["case_axis_perm"],
                            case_axis_sign=md["case_axis_sign"],
                            case_axis_group=md["case_axis_group"],
                            axis_sign_power=md["axis_sign_power"],
                            axis_direction_signs=md["axis_direction_signs"],
                            direction_sign_axis=md["direction_sign_axis"],
                            q_order=q, dim=dim)
                    entry_id, entry_sign = cache[key]
                    if policy["displacement"] == "log2d":
                        disp = (policy["disp_coef"] * scaling
                                * math.log(sbox_extent / table_root_extent)
                                * mode_nmlz[table_lev, sid])
                    else:
                        disp = 0.0
                    integ = table_data[table_lev, entry_id] * entry_sign * scaling + disp
                    acc = acc + coefs[source_id] * integ
            result[target_id] = acc
    return result


def make_list1_case(name, gal, oa, *, dim, q, tree, n_tables, policy, complex_table,
                    complex_coefs, seed, table_root_extent=None, table_starting_level=0,
                    constant_table=False, permute_modes=False, signed=None):
    rng = np.random.default_rng(seed)
    tbl = TableLike(gal, dim, q)
    md = oa.build_arithmetic_case_metadata(tbl, signed)
    n_compact = int(md["n_compact_entries"])
    base = len(range(min(min(v) for v in tbl.interaction_case_vecs),
                     max(max(v) for v in tbl.interaction_case_vecs) + 1))
    shift = -min(min(v) for v in tbl.interaction_case_vecs)
    if constant_table:
        reps = oa.enumerate_scalar_arithmetic_representatives(tbl, md)
        x, w = np.polynomial.legendre.leggauss(q)
        w = 0.5 * w * (table_root_extent or 1.0)
        wt = np.multiply.outer(*([w] * dim)) if dim == 2 else np.multiply.outer(np.multiply.outer(w, w), w)
        wt = wt.reshape(-1)
        smodes = (reps % tbl.n_pairs) // tbl.n_q_points
        table_data = np.tile(wt[smodes], (n_tables, 1))
    elif complex_table:
        table_data = (rng.standard_normal((n_tables, n_compact))
                      + 1j * rng.standard_normal((n_tables, n_compact)))
    else:
        table_data = rng.standard_normal((n_tables, n_compact))
    x, w = np.polynomial.legendre.leggauss(q)
    w = 0.5 * (table_root_extent or 1.0) * w
    nmlz = np.multiply.outer(w, w).reshape(-1) if dim == 2 else np.zeros(q ** dim)
    mode_nmlz = np.tile(nmlz, (n_tables, 1)) * (1.0 + 0.1 * np.arange(n_tables))[:, None]
    if complex_table:
        mode_nmlz = mode_nmlz.astype(np.complex128)
    npts = tree["n_points"]
    if constant_table:
        coefs = np.ones(npts)
    elif complex_coefs:
        coefs = rng.standard_normal(npts) + 1j * rng.standard_normal(npts)
    else:
        coefs = rng.standard_normal(npts)
    nq = q ** dim
    local = np.tile(np.arange(nq, dtype=np.int32), npts // nq)
    smode = local.copy()
    tmode = local.copy()
    if permute_modes:
        # a box-local permutation of the particle order (same for sources/targets)
        perm = rng.permutation(nq).astype(np.int32)
        smode = np.tile(perm, npts // nq)
        tmode = smode.copy()
    tre = table_root_extent if table_root_extent is not None else 1.0
    result = restated_near_field(
        tree, md, oa, q, dim, n_tables, table_data, mode_nmlz, tbl.case_indices,
        base, shift, 1.0e-10, policy, tre, table_starting_level, coefs, smode, tmode)
    np.savez_compressed(
        os.path.join(HERE, f"list1_{name}.npz"),
        dim=np.int64(dim), q=np.int64(q), n_tables=np.int64(n_tables),
        box_centers=tree["box_centers"], box_levels=tree["box_levels"],
        box_starts=tree["box_starts"], box_counts=tree["box_counts"],
        target_boxes=tree["target_boxes"], starts=tree["starts"], lists=tree["lists"],
        root_extent=np.float64(tree["root_extent"]),
        table_root_extent=np.float64(tre), table_starting_level=np.int64(table_starting_level),
        table_data=table_data, mode_nmlz=mode_nmlz, coefs=coefs,
        source_mode_ids=smode, target_point_ids=tmode,
        scaling_exponent=np.int64(policy["scaling_exponent"]),
        displacement=np.array(policy["displacement"]),
        disp_coef=np.float64(policy.get("disp_coef", 0.0)),
        table_level=np.array(policy["table_level"]),
        signed=np.int64(signed is not None),
        result=result)
    print("wrote", name, npts, "points")


def main():
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the volumential source tree>")
    ref_root = sys.argv[1]
    gal = load_ref(ref_root, "list1_gallery")
    oa = load_ref(ref_root, "orbit_arithmetic")

    g2 = gal.generate_list1_gallery(2)
    g3 = gal.generate_list1_gallery(3)
    np.savez_compressed(os.path.join(HERE, "gallery.npz"),
                        vecs2=np.array(g2[0], dtype=np.int64), case_indices2=g2[2],
                        vecs3=np.array(g3[0], dtype=np.int64), case_indices3=g3[2])

    for dim, qs in ((2, (1, 2, 3, 4, 5, 6)), (3, (1, 2, 3, 4, 5))):
        for q in qs:
            tbl = TableLike(gal, dim, q)
            md = oa.build_arithmetic_case_metadata(tbl)
            reps = oa.enumerate_scalar_arithmetic_representatives(tbl, md)
            rows, signs = full_map(oa, md, q, dim, tbl.n_cases)
            save_orbit(os.path.join(HERE, f"orbit_d{dim}_q{q}.npz"), md, reps, rows,
                       signs, seed=100 * dim + q)
            print("orbit", dim, q, md["n_compact_entries"])

    # signed descriptors: target derivative along axis 0 (axis 0 fixed, its own
    # group, odd under reflection), as the reference derives for
    # AxisTargetDerivative(0, Laplace) (orbit_arithmetic.py:177-300)
    for dim, q in ((2, 3), (3, 3)):
        tbl = TableLike(gal, dim, q)
        sym = {"axis_groups": ((0,), tuple(range(1, dim))),
               "axis_sign_power": np.array([1] + [0] * (dim - 1), dtype=np.uint8),
               "axis_direction_signs": np.zeros(dim, dtype=np.int8),
               "direction_sign_axis": -1}
        md = oa.build_arithmetic_case_metadata(tbl, sym)
        reps = oa.enumerate_scalar_arithmetic_representatives(tbl, md)
        rows, signs = full_map(oa, md, q, dim, tbl.n_cases)
        save_orbit(os.path.join(HERE, f"orbit_signed_d{dim}_q{q}.npz"), md, reps, rows,
                   signs, seed=7 + dim)
        print("signed orbit", dim, q, md["n_compact_entries"])

    lap2 = {"scaling_exponent": 2, "displacement": "log2d",
            "disp_coef": -0.5 / 3.141592653589793, "table_level": "zero"}
    lap3 = {"scaling_exponent": 2, "displacement": "none", "table_level": "zero"}
    fixed = {"scaling_exponent": 0, "displacement": "none", "table_level": "zero"}
    perlev = {"scaling_exponent": 0, "displacement": "none", "table_level": "per_level"}

    make_list1_case("lap2d_uniform_l3_q3", gal, oa, dim=2, q=3,
                    tree=uniform_tree(2, 3, 3, -0.5, 0.5), n_tables=1, policy=lap2,
                    complex_table=False, complex_coefs=False, seed=1)
    make_list1_case("lap2d_adaptive_q2", gal, oa, dim=2, q=2,
                    tree=adaptive_tree_2d(2, -0.5, 0.5), n_tables=1, policy=lap2,
                    complex_table=False, complex_coefs=False, seed=2)
    make_list1_case("lap2d_nondyadic_q4", gal, oa, dim=2, q=4,
                    tree=uniform_tree(2, 2, 4, -0.37, 0.91), n_tables=1, policy=lap2,
                    complex_table=False, complex_coefs=False, seed=3,
                    table_root_extent=0.7)
    make_list1_case("lap3d_uniform_l2_q2", gal, oa, dim=3, q=2,
                    tree=uniform_tree(3, 2, 2, -0.5, 0.5), n_tables=1, policy=lap3,
                    complex_table=False, complex_coefs=False, seed=4)
    make_list1_case("lap3d_adaptive_q3", gal, oa, dim=3, q=3,
                    tree=adaptive_tree_3d(3, -0.5, 0.5), n_tables=1, policy=lap3,
                    complex_table=False, complex_coefs=False, seed=5)
    make_list1_case("helm2d_fixed_l3_q3", gal, oa, dim=2, q=3,
                    tree=uniform_tree(2, 3, 3, -0.5, 0.5), n_tables=1, policy=fixed,
                    complex_table=True, complex_coefs=True, seed=6,
                    table_root_extent=0.125, table_starting_level=3)
    make_list1_case("perlevel2d_adaptive_q2", gal, oa, dim=2, q=2,
                    tree=adaptive_tree_2d(2, -0.5, 0.5), n_tables=3, policy=perlev,
                    complex_table=False, complex_coefs=False, seed=7,
                    table_root_extent=0.25, table_starting_level=2)
    make_list1_case("permuted2d_l2_q3", gal, oa, dim=2, q=3,
                    tree=uniform_tree(2, 2, 3, -0.5, 0.5), n_tables=1, policy=lap2,
                    complex_table=False, complex_coefs=False, seed=8, permute_modes=True)
    sym3 = {"axis_groups": ((0,), (1, 2)),
            "axis_sign_power": np.array([1, 0, 0], dtype=np.uint8),
            "axis_direction_signs": np.zeros(3, dtype=np.int8),
            "direction_sign_axis": -1}
    make_list1_case("signed3d_uniform_l2_q2", gal, oa, dim=3, q=2,
                    tree=uniform_tree(3, 2, 2, -0.5, 0.5), n_tables=1,
                    policy={"scaling_exponent": 1, "displacement": "none",
                            "table_level": "zero"},
                    complex_table=False, complex_coefs=False, seed=9, signed=sym3)
    for dim in (2, 3):
        for q in (1, 2):
            make_list1_case(f"constant{dim}d_q{q}", gal, oa, dim=dim, q=q,
                            tree=uniform_tree(dim, 1, q, -1.0, 1.0), n_tables=1,
                            policy={"scaling_exponent": 2, "displacement": "log2d"
                                    if dim == 2 else "none",
                                    "disp_coef": -0.5 / 3.141592653589793,
                                    "table_level": "zero"},
                            complex_table=False, complex_coefs=False, seed=10,
                            table_root_extent=1.0, table_starting_level=1,
                            constant_table=True)


if __name__ == "__main__":
    main()
