"""CPU restatement of the list-1 evaluation with a dense table (numpy, FP64).

TEST INFRASTRUCTURE.  Only ``tests/`` imports this module.  The reference's
dense fallback (``volumential/list1.py:1018-1048``) reads, for each list-1
pair, the table entry of (case, source mode, target point) directly from the
full table; the main loop (``:1050-1159``) adds scaling x entry x source
coefficient over the pair's source points.  Case ids and table levels come
from the C oracle's FP64 case encoding (``OracleProblem.classify_pairs``).
"""

from __future__ import annotations

import numpy as np


def dense_near_field(problem, table_full, *, target_boxes, neighbor_source_boxes_starts,
                     neighbor_source_boxes_lists, box_centers, box_levels, box_starts,
                     box_counts, source_mode_ids, target_point_ids, coefs, root_extent,
                     table_root_extent, scaling_exponent=0):
    """``table_full``: [n_levels, n_cases, nq (source), nq (target)]."""
    cases, levels = problem.classify_pairs(
        target_boxes=target_boxes, neighbor_source_boxes_starts=neighbor_source_boxes_starts,
        neighbor_source_boxes_lists=neighbor_source_boxes_lists, box_centers=box_centers,
        box_levels=box_levels)
    if np.any(cases < 0):
        raise RuntimeError("a list-1 pair falls outside the case gallery")
    coefs = np.asarray(coefs)
    out = np.zeros(len(np.asarray(target_point_ids)),
                   dtype=np.result_type(coefs, table_full))
    for i, tb in enumerate(target_boxes):
        t0, nt = int(box_starts[tb]), int(box_counts[tb])
        tm = np.asarray(target_point_ids[t0:t0 + nt])
        for k in range(neighbor_source_boxes_starts[i], neighbor_source_boxes_starts[i + 1]):
            sb = int(neighbor_source_boxes_lists[k])
            s0, ns = int(box_starts[sb]), int(box_counts[sb])
            sm = np.asarray(source_mode_ids[s0:s0 + ns])
            ext = root_extent * 0.5 ** int(box_levels[sb])
            scaling = (ext / table_root_extent) ** scaling_exponent
            block = table_full[levels[k], cases[k]][np.ix_(sm, tm)]
            out[t0:t0 + nt] += scaling * (coefs[s0:s0 + ns] @ block)
    return out
