"""Arithmetic orbit canonicalisation of near-field table entries (host side).

A full near-field table entry is addressed by ``(case, source mode, target
point)``.  Axis permutations and reflections of the box pair map entries onto
each other; the table stores one value per orbit.  The device kernels never
look up an orbit map: they recompute the compact row of any entry with integer
arithmetic from a few per-case descriptors.  This module builds those
descriptors and enumerates the orbit representatives, restating
``volumential/orbit_arithmetic.py``:

* per-case axis descriptors        -- ``:45-163`` (``_case_arithmetic_axis_descriptors``)
* canonical case of a descriptor   -- ``:166-174``
* compact value count of a case    -- ``:545-563``
* compact row of one entry         -- ``:566-634`` (same arithmetic as the
  generated kernel code ``volumential/list1.py:604-854``)
* case metadata                    -- ``:665-745`` (``build_arithmetic_case_metadata``)
* representative enumeration       -- ``:748-790``

Descriptor semantics (per case ``c`` and output axis ``i``):

``case_axis_perm[c, i]``  input axis feeding output axis ``i``;
``case_axis_sign[c, i]``  -1: reflect (``x -> q-1-x``), +1: keep, 0: the case
                          component is zero and the lexicographically smaller
                          of ``(src, tgt)`` and its reflection is taken;
``case_axis_group[c, i]`` runtime group id; axes of one group are sorted, and
                          each group contributes a multiset rank.
"""

from __future__ import annotations

import itertools
import math

import numpy as np

__all__ = [
    "encode_mode_axes",
    "decode_mode_axes",
    "case_axis_descriptors",
    "canonical_case_vector",
    "compact_case_value_count",
    "rank_sorted_multiset",
    "canonical_entry_axes",
    "evaluate_arithmetic_orbit_entry",
    "evaluate_compact_arithmetic_entry",
    "build_arithmetic_case_metadata",
    "enumerate_scalar_arithmetic_representatives",
    "metadata_nbytes",
]


def encode_mode_axes(axes, q_order):
    """Mode id of per-axis node indices, axis 0 slowest."""
    code = 0
    for a in axes:
        code = code * int(q_order) + int(a)
    return int(code)


def decode_mode_axes(mode_id, q_order, dim):
    """Inverse of :func:`encode_mode_axes`."""
    q = int(q_order)
    out = []
    m = int(mode_id)
    for _ in range(int(dim)):
        out.append(m % q)
        m //= q
    return out[::-1]


def _negating_sign(value):
    # The canonical case vector has non-positive components: a positive
    # component is reflected (-1), a negative one kept (+1), zero marks a
    # self-symmetric axis (0).
    if value > 0:
        return -1
    if value < 0:
        return 1
    return 0


def case_axis_descriptors(case_vec, *, axis_groups=None, direction_signs=None):
    """Return ``(axis_perm u8[dim], axis_sign i8[dim], axis_group u8[dim])``.

    ``axis_groups`` lists the groups of output axes that may be permuted among
    themselves (default: all axes form one group).  ``direction_signs`` (one
    entry per axis, 0 = axis not part of a directional derivative) marks the
    axes of a directional source derivative; those groups use one common
    reflection sign and are resolved by a lexicographic search.
    """
    vec = [int(v) for v in case_vec]
    dim = len(vec)
    groups = (tuple(range(dim)),) if axis_groups is None else axis_groups
    groups = [tuple(sorted(int(a) for a in g)) for g in groups]
    dsign = (np.zeros(dim, dtype=np.int8) if direction_signs is None
             else np.asarray(direction_signs, dtype=np.int8))

    perm = np.zeros(dim, dtype=np.uint8)
    sign = np.zeros(dim, dtype=np.int8)
    group_id = np.zeros(dim, dtype=np.uint8)

    active, inactive = [], []
    for g in groups:
        n_dir = sum(1 for a in g if dsign[a] != 0)
        if n_dir == 0:
            inactive.append(g)
        elif n_dir == len(g):
            active.append(g)
        else:
            raise ValueError("directional arithmetic groups cannot mix active axes")

    next_group = 0
    if active:
        active_axes = sorted(a for g in active for a in g)
        best = None
        for line_sign in (-1, 1):
            for choice in itertools.product(*(itertools.permutations(g) for g in active)):
                cand_perm, cand_sign = {}, {}
                for out_axes, in_axes in zip(active, choice):
                    for o, i in zip(out_axes, in_axes):
                        cand_perm[o] = i
                        cand_sign[o] = line_sign * int(dsign[o]) * int(dsign[i])
                key = (tuple(vec[cand_perm[a]] * cand_sign[a] for a in active_axes),
                       tuple(cand_perm[a] for a in active_axes))
                if best is None or key < best[0]:
                    best = (key, cand_perm, cand_sign)
        _, best_perm, best_sign = best
        for a in active_axes:
            perm[a] = best_perm[a]
            sign[a] = best_sign[a]
            group_id[a] = next_group
            next_group += 1

    for g in inactive:
        # Larger |component| first; ties keep axis order.
        order = sorted(g, key=lambda a: (-abs(vec[a]), a))
        gid = next_group - 1
        prev_abs = None
        for out_axis, in_axis in zip(g, order):
            if abs(vec[in_axis]) != prev_abs:
                gid += 1
                prev_abs = abs(vec[in_axis])
            perm[out_axis] = in_axis
            sign[out_axis] = _negating_sign(vec[in_axis])
            group_id[out_axis] = gid
        next_group = gid + 1

    return perm, sign, group_id


def canonical_case_vector(case_vec, axis_perm, axis_sign):
    """Case vector after applying the descriptors of its case."""
    return [0 if int(s) == 0 else int(case_vec[int(p)]) * int(s)
            for p, s in zip(axis_perm, axis_sign)]


def _n_multisets(alphabet, k):
    return math.comb(int(alphabet) + int(k) - 1, int(k))


def compact_case_value_count(case_axis_sign, case_axis_group, q_order):
    """Number of compact rows stored for one canonical case."""
    signs = np.asarray(case_axis_sign, dtype=np.int64)
    groups = np.asarray(case_axis_group, dtype=np.int64)
    q2 = int(q_order) ** 2
    count = 1
    for g in range(int(groups.max()) + 1):
        members = np.flatnonzero(groups == g)
        if members.size == 0:
            continue
        alphabet = (q2 + 1) // 2 if np.any(signs[members] == 0) else q2
        count *= _n_multisets(alphabet, members.size)
    return int(count)


def rank_sorted_multiset(values, alphabet):
    """Lexicographic rank of a non-decreasing tuple among all multisets."""
    rank = 0
    lo = 0
    k = len(values)
    for pos, v in enumerate(values):
        rest = k - pos - 1
        for c in range(lo, int(v)):
            rank += _n_multisets(int(alphabet) - c, rest)
        lo = int(v)
    return int(rank)


def canonical_entry_axes(case_id, source_mode_id, target_point_id, metadata,
                         q_order, dim):
    """Per-axis (source, target) node indices after reflection/folding and the
    group sort, with the groups, axis signs and entry sign
    (``volumential/orbit_arithmetic.py:372-432`` and the sort of ``:486-507``)."""
    q = int(q_order)
    perm = metadata["case_axis_perm"][case_id]
    signs = metadata["case_axis_sign"][case_id]
    groups = [int(g) for g in metadata["case_axis_group"][case_id]]
    sign_power = metadata["axis_sign_power"]
    dir_signs = metadata["axis_direction_signs"]
    dir_axis = int(metadata["direction_sign_axis"])

    src_raw = decode_mode_axes(source_mode_id, q, dim)
    tgt_raw = decode_mode_axes(target_point_id, q, dim)
    src, tgt = [], []
    entry_sign = 1
    for o in range(dim):
        i = int(perm[o])
        s, t = src_raw[i], tgt_raw[i]
        applied = 1
        if signs[o] < 0:
            s, t, applied = q - 1 - s, q - 1 - t, -1
        elif signs[o] == 0 and (q - 1 - s, q - 1 - t) < (s, t):
            s, t, applied = q - 1 - s, q - 1 - t, -1
        if int(sign_power[i]):
            entry_sign *= applied
        if dir_axis == o:
            entry_sign *= applied * int(dir_signs[i]) * int(dir_signs[o])
        src.append(s)
        tgt.append(t)

    # compare-exchange network over axes of one group: (0,1) in 2D,
    # (0,1), (1,2), (0,1), (0,2) in 3D
    network = [(0, 1)] if dim == 2 else [(0, 1), (1, 2), (0, 1), (0, 2)]
    for a, b in network:
        if groups[a] == groups[b] and (src[b], tgt[b]) < (src[a], tgt[a]):
            src[a], src[b] = src[b], src[a]
            tgt[a], tgt[b] = tgt[b], tgt[a]
    return src, tgt, groups, [int(x) for x in signs], entry_sign


def evaluate_arithmetic_orbit_entry(case_id, source_mode_id, target_point_id,
                                    metadata, q_order, dim):
    """Uncompacted canonical entry id ``orbit * n_pairs + src * nq + tgt`` and
    sign (``volumential/orbit_arithmetic.py:435-515``)."""
    src, tgt, _, _, sign = canonical_entry_axes(
        case_id, source_mode_id, target_point_id, metadata, q_order, dim)
    nq = int(q_order) ** int(dim)
    orbit = int(metadata["case_orbit_ranks"][case_id])
    return (orbit * nq * nq + encode_mode_axes(src, q_order) * nq
            + encode_mode_axes(tgt, q_order)), sign


def evaluate_compact_arithmetic_entry(case_id, source_mode_id, target_point_id,
                                      metadata, q_order, dim):
    """Compact row and sign of one full entry (scalar reference restatement).

    ``metadata`` is the dict returned by :func:`build_arithmetic_case_metadata`.
    Each group of axes contributes the lexicographic rank of its sorted
    multiset of pair codes ``src * q + tgt``; group ranks combine in mixed
    radix; the case orbit's offset is added.
    """
    q = int(q_order)
    src, tgt, groups, signs, entry_sign = canonical_entry_axes(
        case_id, source_mode_id, target_point_id, metadata, q_order, dim)
    q2 = q * q
    compact = 0
    for g in range(max(groups) + 1):
        members = [a for a in range(dim) if groups[a] == g]
        if not members:
            continue
        alphabet = (q2 + 1) // 2 if any(signs[a] == 0 for a in members) else q2
        codes = sorted(src[a] * q + tgt[a] for a in members)
        compact = (compact * _n_multisets(alphabet, len(members))
                   + rank_sorted_multiset(codes, alphabet))
    orbit = int(metadata["case_orbit_ranks"][case_id])
    return int(metadata["case_value_offsets"][orbit]) + compact, entry_sign


def build_arithmetic_case_metadata(table, arithmetic_symmetry=None):
    """Per-case descriptors, orbit ranks and compact offsets of ``table``.

    ``table`` needs ``dim``, ``quad_order``, ``n_cases``,
    ``interaction_case_vecs``, ``case_encode`` and ``case_indices``.
    Returns ``None`` when the compact layout would overflow its integer types
    (the caller then has no arithmetic reconstruction).
    """
    dim = int(table.dim)
    if arithmetic_symmetry is None:
        axis_groups = None
        sign_power = np.zeros(dim, dtype=np.uint8)
        dir_signs = np.zeros(dim, dtype=np.int8)
        dir_axis = -1
    else:
        axis_groups = arithmetic_symmetry["axis_groups"]
        sign_power = np.asarray(arithmetic_symmetry["axis_sign_power"], dtype=np.uint8)
        dir_signs = np.asarray(arithmetic_symmetry["axis_direction_signs"], dtype=np.int8)
        dir_axis = int(arithmetic_symmetry["direction_sign_axis"])

    n_cases = int(table.n_cases)
    perm = np.zeros((n_cases, dim), dtype=np.uint8)
    sign = np.zeros((n_cases, dim), dtype=np.int8)
    group = np.zeros((n_cases, dim), dtype=np.uint8)
    canonical = np.zeros(n_cases, dtype=np.int64)
    for c, vec in enumerate(table.interaction_case_vecs):
        p, s, g = case_axis_descriptors(vec, axis_groups=axis_groups,
                                        direction_signs=dir_signs)
        perm[c], sign[c], group[c] = p, s, g
        canonical[c] = int(table.case_indices[
            table.case_encode(canonical_case_vector(vec, p, s))])

    orbit_cases = np.unique(canonical)
    if orbit_cases.size > np.iinfo(np.uint16).max:
        return None
    orbit_ranks = np.searchsorted(orbit_cases, canonical).astype(np.uint16)

    counts = np.array([compact_case_value_count(sign[c], group[c], table.quad_order)
                       for c in orbit_cases], dtype=np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    if offsets[-1] > np.iinfo(np.int32).max:
        return None

    return {
        "canonical_case_ids": orbit_cases.astype(np.int32),
        "case_orbit_ranks": orbit_ranks,
        "case_axis_perm": perm,
        "case_axis_sign": sign,
        "case_axis_group": group,
        "case_value_offsets": offsets.astype(np.int32),
        "case_value_offsets_i64": offsets,
        "axis_sign_power": sign_power,
        "axis_direction_signs": dir_signs,
        "direction_sign_axis": int(dir_axis),
        "n_compact_entries": int(offsets[-1]),
    }


def enumerate_scalar_arithmetic_representatives(table, metadata):
    """Full entry id stored in each compact row, in row order (int64)."""
    q = int(table.quad_order)
    dim = int(table.dim)
    nq = q ** dim
    q2 = q * q
    out = np.empty(int(metadata["n_compact_entries"]), dtype=np.int64)
    offsets = np.asarray(metadata["case_value_offsets"], dtype=np.int64)
    for rank, case_id in enumerate(np.asarray(metadata["canonical_case_ids"]).tolist()):
        groups = metadata["case_axis_group"][case_id]
        signs = metadata["case_axis_sign"][case_id]
        per_group = []
        for g in range(int(groups.max()) + 1):
            members = [a for a in range(dim) if int(groups[a]) == g]
            if not members:
                continue
            alphabet = (q2 + 1) // 2 if any(int(signs[a]) == 0 for a in members) else q2
            per_group.append(
                (members, list(itertools.combinations_with_replacement(range(alphabet),
                                                                        len(members)))))
        row = int(offsets[rank])
        for combo in itertools.product(*(opts for _, opts in per_group)):
            src = [0] * dim
            tgt = [0] * dim
            for (members, _), codes in zip(per_group, combo):
                for a, code in zip(members, codes):
                    src[a], tgt[a] = divmod(int(code), q)
            out[row] = (int(case_id) * nq * nq + encode_mode_axes(src, q) * nq
                        + encode_mode_axes(tgt, q))
            row += 1
    return out


def metadata_nbytes(metadata):
    """Bytes of the descriptor arrays a kernel reads (reference accounting:
    ``expansion_wrangler_fpnd.py:1699-1708``)."""
    arrays = [metadata["case_orbit_ranks"], metadata["case_axis_perm"],
              metadata["case_axis_sign"], metadata["case_axis_group"],
              metadata["axis_sign_power"], metadata["case_value_offsets"]]
    if int(metadata["direction_sign_axis"]) >= 0:
        arrays.append(metadata["axis_direction_signs"])
    return int(sum(np.asarray(a).nbytes for a in arrays))
