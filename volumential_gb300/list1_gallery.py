"""List-1 interaction gallery: every relative position a list-1 source box can
take with respect to its target box in a 2:1-balanced quadtree/octree.

Follows ``volumential/list1_gallery.py:118-198`` (``generate_interactions``,
``postprocess_interactions``, ``generate_list1_gallery``): the gallery is the
sorted set of integer vectors ``target_center - source_center`` measured on a
grid where a box of the reference level has width 4, over all source boxes of
levels L-1, L, L+1 that touch (l-infinity gap exactly 0) a target box at level L,
plus the zero vector of the self interaction.  The encoding is a base-``base``
positional code of ``vec + shift`` with axis 0 most significant; ``case_indices``
maps a code to its case id and holds -1 for codes that are not list-1 cases.

For ``dim=2`` there are 33 cases with components in [-6, 6] (base 13, shift 6);
for ``dim=3`` there are 139 cases (``case_indices`` has 13**3 = 2197 slots).
"""

from __future__ import annotations

import itertools

import numpy as np

__all__ = ["generate_list1_gallery", "gallery_encoding", "touching_vectors"]


def touching_vectors(dim: int) -> list[tuple[int, ...]]:
    """All ``target_center - source_center`` vectors for touching boxes.

    A complete tree of depth 3 below a root of width 16 is laid out on an
    integer grid (level-2 boxes have width 4).  Target boxes are the level-2
    boxes whose centres lie strictly inside ``(2, 14)`` on every axis, so that
    every neighbour of any size exists.  Source boxes are the boxes of every
    level whose l-infinity gap to the target is exactly zero.
    """
    if dim < 1:
        raise ValueError("dim must be positive")

    boxes = []  # (center vector, half width)
    for level in range(4):
        width = 16 >> level
        half = width // 2
        ticks = np.arange(half, 16, width)
        for center in itertools.product(ticks.tolist(), repeat=dim):
            boxes.append((np.asarray(center, dtype=np.int64), half))

    targets = [
        (c, h) for c, h in boxes
        if h == 2 and int(c.min()) > 2 and int(c.max()) < 14
    ]

    vecs = {tuple([0] * dim)}
    for tc, th in targets:
        for sc, sh in boxes:
            gap = int(np.max(np.abs(tc - sc) - (th + sh)))
            if gap == 0:
                vecs.add(tuple(int(v) for v in (tc - sc)))
    return sorted(vecs)


def gallery_encoding(vec_list):
    """Return ``(base, shift)`` of the positional case code for ``vec_list``."""
    values = sorted({int(v) for vec in vec_list for v in vec})
    lo, hi = values[0], values[-1]
    return hi - lo + 1, -lo


def generate_list1_gallery(dim: int):
    """Return ``(vec_list, case_encode, case_indices)``.

    ``vec_list`` is the lexicographically sorted list of case vectors (case id =
    position in the list), ``case_encode(vec)`` the integer code and
    ``case_indices`` an int64 array of length ``base**dim`` mapping codes to case
    ids (-1 where no case exists).
    """
    vec_list = touching_vectors(dim)
    base, shift = gallery_encoding(vec_list)

    def case_encode(case_vec):
        code = 0
        for comp in case_vec:
            code = code * base + (int(comp) + shift)
        return int(code)

    case_indices = np.full(base ** dim, -1, dtype=np.int64)
    for case_id, vec in enumerate(vec_list):
        case_indices[case_encode(vec)] = case_id

    return vec_list, case_encode, case_indices
