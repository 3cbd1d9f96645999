"""Host-side behaviour of the drop-in API (no GPU needed).

Restates the reference's device-free tests: the scaling-policy strings of
``NearFieldFromCSR`` (test/test_volume_fmm.py:3572-3750) and the
``drive_volume_fmm(list1_only=True)`` contracts with mock wranglers
(test/test_volume_fmm.py:6892-7300), plus the tree builder, the layout
validation and the C ABI library's exported symbols.
"""

import ctypes
import itertools
import os
import re
from types import SimpleNamespace

import numpy as np
import pytest

from volumential_gb300 import _build, _lib
from volumential_gb300.expansion_wrangler_fpnd import (
    _compute_box_local_ids,
    _validate_table_box_particle_layout,
)
from volumential_gb300.expansion_wrangler_interface import ExpansionWranglerInterface
from volumential_gb300.kernels import (
    AxisSourceDerivative,
    AxisTargetDerivative,
    ConstantKernel,
    HelmholtzKernel,
    LaplaceKernel,
)
from volumential_gb300.list1 import (
    NearFieldFromCSR,
    parse_displacement_code,
    parse_policy,
    parse_scaling_code,
    parse_table_level_code,
)
from volumential_gb300.tree_build import (
    build_adaptive_tree,
    build_list1_traversal,
    build_uniform_tree,
)
from volumential_gb300.volume_fmm import drive_volume_fmm

SHAPES1 = {"n_tables": 1, "n_q_points": 1, "n_cases": 1, "n_table_entries": 1}
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# {{{ scaling policy (test/test_volume_fmm.py:3572-3750)

def test_helmholtz_infer_scaling_rejected():
    with pytest.raises(RuntimeError, match="infer_kernel_scaling is unsupported"):
        NearFieldFromCSR(HelmholtzKernel(3), SHAPES1, potential_kind=1,
                         infer_kernel_scaling=True)


def test_policy_per_level_tables_for_helmholtz():
    nf = NearFieldFromCSR(HelmholtzKernel(3), dict(SHAPES1, n_tables=3))
    p = nf.get_kernel_scaling_policy()
    assert p.mode == "per_level_tables"
    assert not p.infer_kernel_scaling and not p.single_table_scaling_supported
    assert p.reference_table_level is None
    assert p.scaling_code == "1.0" and p.displacement_code == "0.0"
    assert "sbox_level" in p.table_level_code
    assert p.scaling_code == nf.codegen_compute_scaling()
    assert p.displacement_code == nf.codegen_compute_displacement()
    assert p.table_level_code == nf.codegen_get_table_level()
    assert parse_policy(p) == {"scaling_exponent": 0, "displacement_kind": 0,
                               "displacement_coef": 0.0,
                               "table_level_kind": _lib.VL1_LEVEL_PER_LEVEL}


def test_policy_fixed_single_table_for_helmholtz():
    nf = NearFieldFromCSR(HelmholtzKernel(3), SHAPES1)
    p = nf.get_kernel_scaling_policy()
    assert p.mode == "fixed_single_table"
    assert p.reference_table_level == 0
    assert (p.scaling_code, p.displacement_code, p.table_level_code) == ("1.0", "0.0", "0.0")
    assert "runtime checks reject mixed source levels" in p.notes
    assert parse_policy(p)["scaling_exponent"] == 0


def test_laplace_derivative_infer_scaling_is_first_order():
    for knl in (AxisTargetDerivative(0, LaplaceKernel(3)),
                AxisSourceDerivative(1, LaplaceKernel(3))):
        nf = NearFieldFromCSR(knl, SHAPES1)
        assert "".join(nf.codegen_compute_scaling().split()) == "sbox_extent/table_root_extent"
        assert parse_scaling_code(nf.codegen_compute_scaling()) == 1


def test_laplace_policy_canonical_table():
    nf = NearFieldFromCSR(LaplaceKernel(2), SHAPES1)
    p = nf.get_kernel_scaling_policy()
    assert p.mode == "canonical_single_table" and p.infer_kernel_scaling
    assert p.single_table_scaling_supported and p.reference_table_level == 0
    assert "sbox_extent" in p.scaling_code
    assert "log(sbox_extent / table_root_extent)" in p.displacement_code
    assert p.table_level_code == "0.0"
    parsed = parse_policy(p)
    assert parsed["scaling_exponent"] == 2
    assert parsed["displacement_kind"] == _lib.VL1_DISP_LOG2D
    assert parsed["displacement_coef"] == pytest.approx(-0.5 / np.pi, rel=1e-15)


def test_custom_scaling_policy_documents_user_code():
    nf = NearFieldFromCSR(HelmholtzKernel(3), SHAPES1, kernel_scaling_code="2 * BOX_extent",
                          kernel_displacement_code="BOX_level")
    p = nf.get_kernel_scaling_policy()
    assert p.mode == "custom_single_table"
    assert p.scaling_code == "2 * sbox_extent"
    assert p.displacement_code == "sbox_level"
    assert p.table_level_code == "0.0"
    with pytest.raises(NotImplementedError):
        parse_policy(p)


def test_policy_memo_follows_extra_kwargs():
    """The per-call plan lookup reuses the parsed policy and cache key until
    the evaluator's extra keyword arguments change."""
    nf = NearFieldFromCSR(LaplaceKernel(3), SHAPES1)
    pol, key = nf._policy_and_key()
    assert key == nf.get_cache_key()
    assert nf._policy_and_key()[1] is key          # memoised
    nf.extra_kwargs["infer_kernel_scaling"] = not nf.extra_kwargs["infer_kernel_scaling"]
    pol2, key2 = nf._policy_and_key()
    assert key2 == nf.get_cache_key() and key2 != key
    assert pol2 == parse_policy(nf.get_kernel_scaling_policy())
    nf.extra_kwargs["list1_precision"] = "mixed"     # any change refreshes the memo
    assert nf._policy_and_key()[1] == nf.get_cache_key()


def test_policy_memo_keys_numpy_scalars_by_value_and_sees_in_place_changes():
    import numpy as np

    nf = NearFieldFromCSR(LaplaceKernel(3), SHAPES1)
    nf.extra_kwargs["some_order"] = np.int64(3)
    key = nf._policy_and_key()[1]
    nf.extra_kwargs["some_order"] = np.int64(3)       # equal value, new object
    assert nf._policy_and_key()[1] is key
    nf.extra_kwargs["some_list"] = [1, 2]
    snap = nf._policy_memo[0]
    nf.extra_kwargs["some_list"].append(3)            # changed in place
    nf._policy_and_key()
    assert nf._policy_memo[0] != snap
    obj = object()
    nf.extra_kwargs["some_object"] = obj
    nf._policy_and_key()
    assert any(v is obj for v in nf._policy_memo[3])   # held: its id cannot be reused


def test_laplace_2d_derivative_has_no_log_displacement():
    for knl in (AxisTargetDerivative(0, LaplaceKernel(2)),
                AxisSourceDerivative(1, LaplaceKernel(2))):
        nf = NearFieldFromCSR(knl, SHAPES1)
        assert "".join(nf.codegen_compute_displacement().split()) == "0.0"


def test_constant_kernel_scaling_codes():
    assert parse_scaling_code(NearFieldFromCSR(ConstantKernel(3), SHAPES1)
                              .codegen_compute_scaling()) == 3
    assert parse_scaling_code(NearFieldFromCSR(ConstantKernel(2), SHAPES1)
                              .codegen_compute_scaling()) == 2


def test_helmholtz_split_policy_codes_parse():
    """The split rules of expansion_wrangler_fpnd.py:4777-4833."""
    assert parse_scaling_code("(sbox_extent * sbox_extent) / "
                              "(table_root_extent * table_root_extent)") == 2
    assert parse_scaling_code("(table_root_extent) / (sbox_extent)") == -1
    kind, coef = parse_displacement_code(
        f"-0.5 / {np.pi!r} * scaling * log(sbox_extent / table_root_extent) * "
        "mode_nmlz[table_lev, sid]")
    assert kind == _lib.VL1_DISP_LOG2D and coef == pytest.approx(-0.5 / np.pi)
    assert parse_table_level_code("0.0") == _lib.VL1_LEVEL_ZERO


def test_batch_size_must_be_positive():
    nf = NearFieldFromCSR(LaplaceKernel(2), SHAPES1, list1_target_batch_size=0)
    with pytest.raises(ValueError, match="must be positive"):
        nf._target_batch_size()


def test_vec_id_code_matches_reference_form():
    nf = NearFieldFromCSR(LaplaceKernel(2), SHAPES1)
    code = nf.codegen_vec_id()
    assert code.startswith("((0.0) * encoding_base+((box_centers[0, target_box_id]")
    assert "/ sbox_extent * 4.0 + encoding_shift + 1e-10" in code

# }}}


# {{{ drive_volume_fmm contracts (test/test_volume_fmm.py:6892-7300)

class _MockWrangler(ExpansionWranglerInterface):
    dtype = np.float64

    def __init__(self, out=None, source_map=None):
        self._out = out
        self._source_map = source_map
        self.reordered_src_weights = None
        self.reordered_src_func = None

    def output_zeros(self):
        return np.array([0.0])

    def reorder_sources(self, source_array):
        src = np.asarray(source_array)
        return src if self._source_map is None else src[self._source_map]

    def reorder_potentials(self, potentials):
        return potentials

    def form_multipoles(self, level_start_source_box_nrs, source_boxes, src_weights):
        self.reordered_src_weights = np.asarray(src_weights[0]).copy()
        return None, None

    def coarsen_multipoles(self, a, b, mpoles):
        return mpoles, None

    def eval_direct(self, target_boxes, starts, lists, mode_coefs):
        self.reordered_src_func = np.asarray(mode_coefs).copy()
        if self._out is not None:
            return self._out.copy(), None
        return np.array([np.sum(mode_coefs)]), None

    def finalize_potentials(self, potentials):
        return potentials


def _traversal(ns=3, nt=5):
    e = np.array([], dtype=np.int32)
    return SimpleNamespace(
        tree=SimpleNamespace(nsources=ns, ntargets=nt, sources_are_targets=True),
        level_start_source_box_nrs=e, source_boxes=e, level_start_source_parent_box_nrs=e,
        source_parent_boxes=e, target_boxes=e, neighbor_source_boxes_starts=e,
        neighbor_source_boxes_lists=e)


def test_list1_multi_source_superposition():
    src0 = np.array([1.0, 2.0, 3.0])
    src1 = np.array([10.0, 20.0, 30.0])
    sw = np.empty(2, dtype=object)
    sw[:] = [src0, src1]
    sf = np.empty(2, dtype=object)
    sf[:] = [src0, src1]
    result = drive_volume_fmm(_traversal(), _MockWrangler(), sw, sf, list1_only=True)
    if isinstance(result, np.ndarray) and result.dtype == object:
        result = result[0]
    assert np.allclose(result, [66.0])


def test_rejects_mismatched_source_field_counts():
    src0 = np.array([1.0, 2.0, 3.0])
    sw = np.empty(2, dtype=object)
    sw[:] = [src0, 10 * src0]
    with pytest.raises(ValueError, match="same field count"):
        drive_volume_fmm(_traversal(3, 3), _MockWrangler(), sw, src0)


def test_reorders_src_func_with_source_permutation():
    w = _MockWrangler(source_map=np.array([2, 0, 1]))
    result = drive_volume_fmm(_traversal(), w, np.array([1.0, 2.0, 4.0]),
                              np.array([10.0, 20.0, 40.0]), list1_only=True)
    assert np.allclose(w.reordered_src_weights, [4.0, 1.0, 2.0])
    assert np.allclose(w.reordered_src_func, [40.0, 10.0, 20.0])
    assert np.allclose(result, [70.0])


def test_nonfinite_list1_values_raise():
    w = _MockWrangler(out=np.array([np.nan, 1.0]))
    with pytest.raises(RuntimeError, match="non-finite values"):
        drive_volume_fmm(_traversal(3, 2), w, np.array([1.0, 2.0, 3.0]),
                         np.array([10.0, 20.0, 30.0]), list1_only=True)


def test_rejects_removed_p2p_fallback_option():
    with pytest.raises(TypeError, match="allow_list1_p2p_fallback"):
        drive_volume_fmm(_traversal(), _MockWrangler(), np.ones(3), np.ones(3),
                         list1_only=True, allow_list1_p2p_fallback=True)


def test_non_list1_drive_is_not_implemented():
    with pytest.raises(NotImplementedError, match="list1_only"):
        drive_volume_fmm(_traversal(), _MockWrangler(), np.ones(3), np.ones(3))

# }}}


# {{{ tree builder and layout checks

def _brute_list1(tree):
    ext = tree.root_extent / 2.0 ** tree.box_levels.astype(float)
    out = {}
    for t in tree.leaf_boxes:
        gap = np.max(np.abs(tree.box_centers[:, tree.leaf_boxes]
                            - tree.box_centers[:, [t]])
                     - 0.5 * (ext[tree.leaf_boxes] + ext[t])[None, :], axis=0)
        out[int(t)] = sorted(int(s) for s in tree.leaf_boxes[gap < 1e-12])
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_list1_csr_matches_brute_force(dim):
    rng = np.random.default_rng(dim)
    centers = rng.uniform(-0.5, 0.5, (3, dim))

    def refine(nodes):
        v = sum(np.exp(-np.sum((nodes - c[:, None, None]) ** 2, axis=0) / 0.05 ** 2)
                for c in centers)
        return (v.max(-1) - v.min(-1)) > 1e-3

    for tree in (build_uniform_tree(dim, 2, 2),
                 build_adaptive_tree(dim, 2, refine, max_level=6 if dim == 2 else 4,
                                     min_level=2)):
        trav = build_list1_traversal(tree)
        ref = _brute_list1(tree)
        st = trav.neighbor_source_boxes_starts
        for i, t in enumerate(trav.target_boxes):
            got = trav.neighbor_source_boxes_lists[st[i]:st[i + 1]].tolist()
            assert got == ref[int(t)]
            lv = tree.box_levels.astype(int)
            assert np.all(np.abs(lv[got] - lv[t]) <= 1)


def test_uniform_tree_sizes():
    tree = build_uniform_tree(2, 5, 4)
    trav = build_list1_traversal(tree)
    assert tree.ntargets == 16384 and len(trav.target_boxes) == 1024
    assert tree.nboxes == 1365 and tree.aligned_nboxes % 32 == 0
    assert trav.nnz == (3 * 32 - 2) ** 2
    assert np.all(tree.box_levels[trav.target_boxes] == 5)


def test_leaf_nodes_are_gauss_legendre_in_ij_order():
    tree = build_uniform_tree(2, 1, 3, a=0.0, b=2.0)
    x, w = np.polynomial.legendre.leggauss(3)
    leaf = tree.leaf_boxes[0]
    pts = tree.targets[:, tree.box_target_starts[leaf]:tree.box_target_starts[leaf] + 9]
    c = tree.box_centers[:, leaf]
    gx, gy = np.meshgrid(c[0] + 0.5 * x, c[1] + 0.5 * x, indexing="ij")
    assert np.allclose(pts[0], gx.ravel()) and np.allclose(pts[1], gy.ravel())
    assert np.isclose(tree.weights.sum(), 4.0)


def test_box_local_ids_and_layout_validation():
    tree = build_uniform_tree(2, 2, 2)
    trav = build_list1_traversal(tree)
    local = _compute_box_local_ids(tree, 4)
    assert np.array_equal(local[:8], [0, 1, 2, 3, 0, 1, 2, 3])
    _validate_table_box_particle_layout(tree, trav.target_boxes,
                                        trav.neighbor_source_boxes_lists, 4)
    with pytest.raises(ValueError, match="requires exactly"):
        _validate_table_box_particle_layout(tree, trav.target_boxes,
                                            trav.neighbor_source_boxes_lists, 9)
    with pytest.raises(ValueError, match="not divisible"):
        _compute_box_local_ids(tree, 3)

# }}}


# {{{ the C ABI library

def _header_functions():
    with open(os.path.join(ROOT, "include", "vl1.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|int64_t|const char \*)\s*(vl1_\w+)\(",
                                 text, flags=re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    path = _build.build()
    lib = ctypes.CDLL(path)
    declared = _header_functions()
    assert len(declared) >= 8
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_lib.SIGNATURES)
    handle = _lib.lib()
    assert handle.vl1_version() >= 100


def test_capi_rejects_bad_plan_descriptions_without_a_gpu():
    lib = _lib.lib()
    d = _lib.PlanDesc()
    d.dim = 4
    out = ctypes.c_void_p()
    assert lib.vl1_plan_create(ctypes.byref(d), ctypes.byref(out)) == _lib.VL1_E_UNSUPPORTED
    assert b"dim" in lib.vl1_last_error_string()
    d.dim = 2
    d.reconstruction_kind = 7
    assert lib.vl1_plan_create(ctypes.byref(d), ctypes.byref(out)) == \
        _lib.VL1_E_UNSUPPORTED_RECON
    assert lib.vl1_plan_create(None, ctypes.byref(out)) == _lib.VL1_E_ARG
    assert lib.vl1_eval_fp64(None, None, None, 0, 1, None, None) == _lib.VL1_E_ARG

# }}}


def test_mixed_work_items_cover_every_key_once():
    from volumential_gb300.batched import MixedSchedule

    rng = np.random.default_rng(5)
    counts = rng.integers(0, 40, size=60)
    counts[3] = 0
    key_start = np.concatenate([[0], np.cumsum(counts)])
    for cap in (1, 3, 8, 1000):
        items, n_splits, n_slots = MixedSchedule._work_items(key_start, cap)
        lens = [it[2] - it[1] for it in items]
        assert lens == sorted(lens, reverse=True)
        assert max(lens) <= cap
        covered = np.zeros(int(key_start[-1]), dtype=int)
        slots = set()
        parts = {}
        for tile, k0, k1, split, part, nparts, slot, _ in items:
            assert key_start[tile] <= k0 <= k1 <= key_start[tile + 1]
            covered[k0:k1] += 1
            if split < 0:
                assert (part, nparts, slot) == (0, 1, -1)
                assert (k0, k1) == (key_start[tile], key_start[tile + 1])
            else:
                assert 0 <= part < nparts and 0 <= slot < n_slots
                slots.add(slot)
                parts.setdefault(split, []).append((part, slot, tile))
        assert np.all(covered == 1)
        assert len(slots) == n_slots and len(parts) == n_splits
        for split, ps in parts.items():
            ps.sort()
            assert [p for p, _, _ in ps] == list(range(len(ps)))
            assert len({t for _, _, t in ps}) == 1
            base = ps[0][1]
            assert [s for _, s, _ in ps] == list(range(base, base + len(ps)))


def _pack_rows_by_loop(mask, rows_per_tile):
    """Plain-Python restatement of the greedy tile packing (test only)."""
    sigs = {}
    for b in range(mask.shape[0]):
        sigs.setdefault(tuple(np.flatnonzero(mask[b])), []).append(b)
    # signature order of np.unique over the packed little-endian words
    def word_key(sig):
        words = [0] * (-(-mask.shape[1] // 64))
        for k in map(int, sig):
            words[k // 64] |= 1 << (k % 64)
        return tuple(words)
    order_sigs = sorted(sigs, key=word_key)
    groups = [list(sigs[g]) for g in order_sigs]
    keysets = [set(g) for g in order_sigs]
    out = []
    while any(groups):
        tile, space = set(), rows_per_tile
        s_ = max(range(len(groups)), key=lambda i: (len(groups[i]), -i))
        while True:
            take = min(space, len(groups[s_]))
            out += groups[s_][:take]
            groups[s_] = groups[s_][take:]
            space -= take
            tile |= keysets[s_]
            if space == 0 or not any(groups):
                break
            best = None
            for i, g in enumerate(groups):
                if not g:
                    continue
                score = len(keysets[i] - tile) / max(min(len(g), space), 1)
                cand = (score, -len(g), i)
                if best is None or cand < best:
                    best = cand
            s_ = best[2]
    return np.array(out)


def _tile_schedule_by_loop(keys, starts, lists, n_tb, K, nrhs):
    """Straightforward per-tile restatement of the tile schedule (test only)."""
    tb_of_pair = np.repeat(np.arange(n_tb), np.diff(starts))
    mask = np.zeros((n_tb, K), dtype=bool)
    mask[tb_of_pair, keys] = True
    order = _pack_rows_by_loop(mask, max(1, 128 // nrhs))
    rows = (order[:, None] * nrhs + np.arange(nrhs)[None, :]).ravel()
    n_tiles = (len(rows) + 127) // 128
    tile_rows = np.full(n_tiles * 128, -1)
    tile_rows[:len(rows)] = rows
    tile_rows = tile_rows.reshape(n_tiles, 128)
    src = {(int(tb_of_pair[p]), int(keys[p])): int(lists[p]) for p in range(len(keys))}
    tiles = []
    for t in range(n_tiles):
        js = [int(v) // nrhs for v in tile_rows[t] if v >= 0]
        tkeys = sorted({int(keys[p]) for j in set(js) for p in range(starts[j], starts[j + 1])})
        xr = []
        for k in tkeys:
            row = []
            for v in tile_rows[t]:
                s_ = src.get((int(v) // nrhs, k)) if v >= 0 else None
                row.append(-1 if s_ is None else s_ * nrhs + int(v) % nrhs)
            xr.append(row)
        tiles.append((tkeys, xr))
    lpt = sorted(range(n_tiles), key=lambda t: -len(tiles[t][0]))
    key_start, key_ids, xrow = [0], [], []
    for t in lpt:
        key_ids += tiles[t][0]
        xrow += tiles[t][1]
        key_start.append(len(key_ids))
    return tile_rows[lpt], np.array(key_start), np.array(key_ids), np.array(xrow).reshape(-1, 128)


@pytest.mark.parametrize("K", [40, 139, 300])
def test_pack_rows_matches_the_greedy_restatement_and_packs_tighter(K):
    from volumential_gb300.batched import MixedSchedule

    rng = np.random.default_rng(K)
    n_tb = 700
    # boxes drawn from a few dozen signatures, as on a tree
    protos = [rng.choice(K, size=rng.integers(3, 12), replace=False) for _ in range(40)]
    mask = np.zeros((n_tb, K), dtype=bool)
    for b in range(n_tb):
        mask[b, protos[rng.integers(len(protos))]] = True
    got = MixedSchedule.pack_rows(mask, 128)
    assert np.array_equal(np.sort(got), np.arange(n_tb))
    assert np.array_equal(got, _pack_rows_by_loop(mask, 128))

    def tile_keys(order):
        return sum(mask[order[i:i + 128]].any(axis=0).sum() for i in range(0, n_tb, 128))
    _, sig = np.unique(np.packbits(mask, axis=1), axis=0, return_inverse=True)
    assert tile_keys(got) <= tile_keys(np.lexsort((np.arange(n_tb), sig.ravel())))


@pytest.mark.parametrize("nrhs", [1, 3, 130])
def test_tile_schedule_matches_per_tile_restatement(nrhs):
    from volumential_gb300.batched import MixedSchedule

    rng = np.random.default_rng(11 + nrhs)
    n_tb, K = 300, 40
    deg = rng.integers(0, 9, size=n_tb)
    starts = np.concatenate([[0], np.cumsum(deg)])
    keys = np.concatenate([rng.choice(K, size=d, replace=False) for d in deg]).astype(np.int64)
    lists = rng.integers(0, 500, size=len(keys)).astype(np.int64)
    got = MixedSchedule.tile_schedule(keys, starts, lists, n_tb, K, nrhs)
    want = _tile_schedule_by_loop(keys, starts, lists, n_tb, K, nrhs)
    for g, w in zip(got, want):
        assert np.array_equal(np.asarray(g), np.asarray(w))


# restatement of the work-item cost model of vl1_mixed_work_items (test only)
ITEM_OVERHEAD_KEYS, SPLIT_OVERHEAD_KEYS, LAST_PART_KEYS = 4.0, 1.5, 2.0
CAP_FRACTIONS = (1.5, 1.25, 1.0, 0.85, 0.75, 0.67, 0.6, 0.5, 0.4, 0.33, 0.25, 0.2, 0.17)


def _split_items(key_start, cap):
    items, n_splits, n_slots = [], 0, 0
    for t in range(len(key_start) - 1):
        k0, k1 = int(key_start[t]), int(key_start[t + 1])
        nk = k1 - k0
        nparts = max(1, -(-nk // cap))
        if nparts == 1:
            items.append((t, k0, k1, -1, 0, 1, -1, 0))
            continue
        bounds = [k0 + (nk * i) // nparts for i in range(nparts + 1)]
        for part in range(nparts):
            items.append((t, bounds[part], bounds[part + 1], n_splits, part, nparts,
                          n_slots + part, 0))
        n_splits += 1
        n_slots += nparts
    items.sort(key=lambda it: -(it[2] - it[1]))
    return items, n_splits, n_slots


def test_work_item_cap_choice_equals_the_exhaustive_search():
    """The cap search skips candidates whose lower bound cannot beat the best
    so far and uses max(cost) when every item has its own slot; the chosen
    work list is the one an exhaustive search over the candidates picks."""
    import heapq

    from volumential_gb300.batched import MixedSchedule as M

    def finish(items, n_sm):
        slots = [0.0] * n_sm
        for it in items:
            cost = (it[2] - it[1]) + ITEM_OVERHEAD_KEYS
            if it[3] >= 0:
                cost += SPLIT_OVERHEAD_KEYS + (LAST_PART_KEYS if it[4] == it[5] - 1 else 0)
            heapq.heapreplace(slots, slots[0] + cost)
        return max(slots)

    rng = np.random.default_rng(21)
    for _ in range(60):
        nt = int(rng.integers(1, 300))
        ks = np.concatenate([[0], np.cumsum(rng.integers(1, 80, size=nt))])
        n_sm = int(rng.integers(1, 160))
        share = max(1, -(-int(ks[-1]) // n_sm))
        best = None
        for f in CAP_FRACTIONS:
            cand = _split_items(ks, max(4, int(np.ceil(share * f))))
            t = finish(cand[0], n_sm)
            if best is None or t < best[0]:
                best = (t, cand)
        def as_tuples(r):
            return [tuple(int(v) for v in row) for row in r[0]], r[1], r[2]
        assert as_tuples(M._work_items(ks, None, n_sm=n_sm)) == best[1]
        cap = int(rng.integers(1, 60))
        assert as_tuples(M._work_items(ks, cap, n_sm=n_sm)) == _split_items(ks, cap)


def test_tile_schedule_rejects_two_sources_with_one_case():
    from volumential_gb300.batched import MixedSchedule

    starts = np.array([0, 2])
    with pytest.raises(RuntimeError):
        MixedSchedule.tile_schedule(np.array([3, 3]), starts, np.array([1, 2]), 1, 5, 1)


# ---- serving: resident budget and the C5 mix (host logic) -----------------

def test_resident_budget_evicts_idle_entries_oldest_first():
    from volumential_gb300.serving import AdmissionError, ResidentBudget

    released = []
    b = ResidentBudget(100, release_fn=released.append)
    b.admit("a", 40, lambda: "A")
    b.admit("b", 40, lambda: "B")
    b.get("a")                      # "a" is now the most recently used
    b.admit("c", 40, lambda: "C")   # evicts "b", the least recently used
    assert released == ["B"] and "a" in b and "c" in b and b.used == 80
    b.pin("a")
    b.pin("c")
    with pytest.raises(AdmissionError):
        b.admit("d", 40, lambda: "D")   # both residents busy
    assert "d" not in b and b.used == 80
    b.unpin("c")
    b.admit("d", 40, lambda: "D")
    assert released == ["B", "C"] and b.evictions == 2
    with pytest.raises(AdmissionError):
        b.admit("e", 101, lambda: "E")  # larger than the whole budget
    b.resize("d", 10)
    assert b.used == 50 and b.make_room(50) and not b.make_room(101)


def test_c5_mix_follows_its_sampling_rules():
    from volumential_gb300.workloads import _nearest_level, config_c5, poisson_arrivals

    probs, reqs, mixes = config_c5(n_requests=400)
    probs2, reqs2, _ = config_c5(n_requests=400)
    assert reqs == reqs2 and sorted(probs) == sorted(probs2)
    assert len(reqs) == 400 and set(k for k, _ in reqs) <= set(probs)
    assert 400 < len(probs) < 800   # catalogue draws; Laplace draws repeat problems
    dims = [k[0] for k, _ in reqs]
    kerns = [k[1] for k, _ in reqs]
    assert 0.4 < dims.count(2) / 400 < 0.6 and 0.4 < kerns.count("laplace") / 400 < 0.6
    for key, p in probs.items():
        assert p.n_points == (2 ** p.dim) ** p.level * p.q ** p.dim
        assert p.q in (3, 4, 5)
        assert (p.k == 0) == (p.kernel == "laplace")
        assert p.kernel == "laplace" or 1 <= p.k <= 30
        assert p.table_key == ((p.dim, p.kernel, 0.0, p.q) if p.kernel == "laplace"
                               else (p.dim, p.kernel, p.k, p.q, p.level))
        assert len(mixes[key]) == 4
    # k is drawn from the real interval, not its integers
    ks = [p.k for p in probs.values() if p.kernel == "helmholtz"]
    assert len(set(ks)) == len(ks) and any(k != int(k) for k in ks)
    # nearest level in log: 2D q4 N=5000 -> level 4 (4096), 3D q3 N=3e5 -> 4 (110,592)
    assert _nearest_level(2, 4, 5000) == 4 and _nearest_level(3, 3, 3e5) == 4
    t = poisson_arrivals(20000, 1000.0, seed=1)
    assert np.all(np.diff(t) > 0) and abs(t[-1] / 20000 - 1e-3) < 5e-5


def test_header_constants_match_the_python_binding():
    """Every enumerator and integer #define of include/vl1.h has the same value
    in the ctypes binding (status codes, dtypes, policy and builder codes,
    split flags, the no-alloc scratch size)."""
    import os
    import re

    from volumential_gb300 import _lib

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    text = open(os.path.join(root, "include", "vl1.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    consts = {}
    for body in re.findall(r"enum\s*\{(.*?)\}", text, flags=re.S):
        for name, val in re.findall(r"(VL1_[A-Z0-9_]+)\s*=\s*([^,\s]+)", body):
            consts[name] = int(val, 0)
    for name, a, b in re.findall(r"#define\s+(VL1_[A-Z0-9_]+)\s+\((\d+)LL\s*<<\s*(\d+)\)", text):
        consts[name] = int(a) << int(b)
    for name, val in re.findall(r"#define\s+(VL1_[A-Z0-9_]+)\s+(\d+)\s*$", text, flags=re.M):
        consts[name] = int(val)
    assert len(consts) >= 28
    for name, val in consts.items():
        assert getattr(_lib, name) == val, name


def test_dense_fallback_takes_full_tables_only():
    # list1.py:1018-1048: a kernel without the arithmetic orbit symmetry
    # keeps a full table; a symmetry-reduced one would need the
    # generated-orbit fallback, which is not built
    import numpy as np
    import pytest

    from volumential_gb300.expansion_wrangler_fpnd import _prepare_table_data_and_entry_map
    from volumential_gb300.kernels import PlaneWaveKernel
    from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

    t = NearFieldInteractionTable(2, dim=2, sumpy_kernel=PlaneWaveKernel(2),
                                  source_box_extent=0.5)
    assert t._get_invariant_entry_info() is None
    rng = np.random.default_rng(0)
    t.data = rng.standard_normal(t.n_cases * t.n_pairs)
    tdc, nm, ext, ids, scales, info = _prepare_table_data_and_entry_map([t, t])
    assert info["kind"] == "dense" and tdc.shape == (2, t.n_cases * t.n_pairs)
    assert np.array_equal(tdc[1], t.data) and np.array_equal(ids, np.arange(tdc.shape[1]))
    t.set_reduced_table_data(np.arange(10), np.ones(10))
    with pytest.raises(NotImplementedError):
        _prepare_table_data_and_entry_map([t])


def test_derivative_kernels_take_the_signed_arithmetic_symmetry():
    # orbit_arithmetic.py:176-300: differentiated axes fixed (own groups) and
    # odd under reflection, the other axes one group
    import numpy as np

    from volumential_gb300.kernels import (
        AxisSourceDerivative,
        AxisTargetDerivative,
        LaplaceKernel,
        PlaneWaveKernel,
        arithmetic_symmetry,
    )

    assert arithmetic_symmetry(LaplaceKernel(3), 3) is None
    assert arithmetic_symmetry(PlaneWaveKernel(2), 2) is False
    s = arithmetic_symmetry(AxisTargetDerivative(1, LaplaceKernel(3)), 3)
    assert s["axis_groups"] == ((1,), (0, 2))
    assert np.array_equal(s["axis_sign_power"], [0, 1, 0])
    s2 = arithmetic_symmetry(AxisSourceDerivative(0, AxisTargetDerivative(0, LaplaceKernel(2))), 2)
    assert s2["axis_groups"] == ((0,), (1,)) and np.array_equal(s2["axis_sign_power"], [0, 0])
    s3 = arithmetic_symmetry(AxisSourceDerivative(2, AxisTargetDerivative(0, LaplaceKernel(3))), 3)
    assert s3["axis_groups"] == ((0,), (2,), (1,))
    assert np.array_equal(s3["axis_sign_power"], [1, 0, 1])
