"""``drive_volume_fmm`` -- the list-1 stage (``list1_only=True``) on GB300.

Restates ``volumential/volume_fmm.py:677-1053`` for the list-1 path:

* source-field normalisation (``:174-208``, ``:729-745``) and the field-count
  check;
* rejection of the removed ``allow_list1_p2p_fallback`` option (``:750-754``);
* reordering of every field into tree order (``:869-873``);
* the multipole stages are called as in the reference (their result is not
  used by a ``list1_only`` drive);
* list 1 per field with a non-finite check that raises (``:983-995``), then
  superposition of the fields (``:1028-1031``);
* ``reorder_potentials`` / ``finalize_potentials`` and return (``:1040-1053``).

A wrangler that offers ``eval_direct_batched`` evaluates all fields in one
launch; the result is the same sum of per-field potentials.  Stages outside
list 1 (far field, global direct evaluation,
target interpolation) raise ``NotImplementedError``.
"""

from __future__ import annotations

import logging

import numpy as np

logger = logging.getLogger(__name__)

__all__ = ["drive_volume_fmm"]


def _is_tensor(x):
    return hasattr(x, "data_ptr") and hasattr(x, "dim")


def _normalize_source_fields(values, dtype, *, expected_length=None, field_name="source"):
    """List of fields (1D arrays) from an object array, a list, a 1D or 2D array."""
    if isinstance(values, np.ndarray) and values.dtype == object:
        if values.ndim > 1:
            raise ValueError(f"{field_name} must be 1D or 2D, got ndim={values.ndim}")
        fields = list(values.flat)
    elif isinstance(values, (list, tuple)):
        arr = None
        if values and not any(_is_tensor(v) for v in values):
            arr = np.asarray(values)
        if arr is not None and arr.ndim == 1 and arr.dtype != object:
            fields = [arr]
        elif arr is not None and arr.ndim == 2 and arr.dtype != object:
            fields = [arr[i] for i in range(arr.shape[0])]
        else:
            fields = list(values)
    elif hasattr(values, "ndim") and values.ndim == 2:
        if expected_length is not None and values.shape[0] == expected_length \
                and values.shape[1] != expected_length:
            fields = [values[:, i] for i in range(values.shape[1])]
        else:
            fields = [values[i] for i in range(values.shape[0])]
    elif hasattr(values, "ndim") and values.ndim > 2:
        raise ValueError(f"{field_name} must be 1D or 2D, got ndim={values.ndim}")
    else:
        fields = [values]
    out = np.empty(len(fields), dtype=object)
    for i, f in enumerate(fields):
        out[i] = f
    return out


def _contains_nonfinite(values):
    if isinstance(values, (list, tuple)) or (
            isinstance(values, np.ndarray) and values.dtype == object):
        items = list(values)
    else:
        items = [values]
    for v in items:
        if _is_tensor(v):
            import torch
            if not bool(torch.isfinite(v).all()):
                return True
        else:
            a = np.asarray(v)
            if np.isnan(a).any() or np.isinf(a).any():
                return True
    return False


def _add(a, b):
    if isinstance(a, list):
        return [x + y for x, y in zip(a, b)]
    return a + b


def drive_volume_fmm(traversal, expansion_wrangler, src_weights, src_func,
                     direct_evaluation=False, timing_data=None, reorder_sources=True,
                     reorder_potentials=True, **kwargs):
    """Volume potential driver; only the list-1 stage is implemented.

    Returns the list-1 potentials of the superposed source fields, in user
    order when ``reorder_potentials`` is true.
    """
    wrangler = expansion_wrangler
    dtype = getattr(wrangler, "dtype", np.float64)
    expected = None
    if hasattr(traversal, "tree"):
        expected = getattr(traversal.tree, "nsources", None)
        if expected is None:
            expected = getattr(traversal.tree, "ntargets", None)

    src_weights = _normalize_source_fields(src_weights, dtype, expected_length=expected,
                                           field_name="src_weights")
    src_func = _normalize_source_fields(src_func, dtype, expected_length=expected,
                                        field_name="src_func")
    ns = len(src_weights)
    if ns != len(src_func):
        raise ValueError("src_weights and src_func must have the same field count")

    list1_only = bool(kwargs.get("list1_only", False))
    kwargs.pop("auto_interpolate_targets", None)
    if "allow_list1_p2p_fallback" in kwargs:
        raise TypeError(
            "drive_volume_fmm no longer accepts allow_list1_p2p_fallback; "
            "non-finite list1 table results now raise an error")
    if direct_evaluation:
        raise NotImplementedError("global direct (P2P) evaluation is not part of the "
                                  "GB300 list-1 path")
    if not list1_only:
        raise NotImplementedError(
            "only the list-1 stage is implemented on GB300: call with list1_only=True")

    if reorder_sources:
        for i in range(ns):
            src_weights[i] = wrangler.reorder_sources(src_weights[i])
            src_func[i] = wrangler.reorder_sources(src_func[i])

    mpole_exps, _ = wrangler.form_multipoles(
        getattr(traversal, "level_start_source_box_nrs", None),
        getattr(traversal, "source_boxes", None), src_weights)
    wrangler.coarsen_multipoles(
        getattr(traversal, "level_start_source_parent_box_nrs", None),
        getattr(traversal, "source_parent_boxes", None), mpole_exps)

    split = bool(getattr(wrangler, "helmholtz_split", False)) and \
        hasattr(wrangler, "eval_direct_helmholtz_split_correction")

    def split_correction(idx, field_pot):
        """volume_fmm.py:999-1026: add the split mode's list-1 remainder."""
        corr, _ = wrangler.eval_direct_helmholtz_split_correction(
            traversal.target_boxes, traversal.neighbor_source_boxes_starts,
            traversal.neighbor_source_boxes_lists, src_weights[idx], src_func=src_func[idx])
        if _contains_nonfinite(corr):
            raise RuntimeError("Helmholtz split list1 correction produced non-finite values "
                               f"for field {idx}")
        out = [p + c for p, c in zip(field_pot, corr)]
        if _contains_nonfinite(out):
            raise RuntimeError("combined list1 potential produced non-finite values after "
                               f"Helmholtz split correction for field {idx}")
        return out

    potentials = None
    batched = getattr(wrangler, "eval_direct_batched", None)
    if batched is not None and ns > 1:
        import torch

        from .plan import as_device_tensor
        stacked = torch.stack([as_device_tensor(f) for f in src_func])
        per_kernel, _ = batched(traversal.target_boxes,
                                traversal.neighbor_source_boxes_starts,
                                traversal.neighbor_source_boxes_lists, stacked)
        for idx in range(ns):
            field_pot = [p[idx] for p in per_kernel]
            if _contains_nonfinite(field_pot):
                raise RuntimeError(
                    "table-based list1 evaluation produced non-finite values for "
                    f"field {idx}; check near-field table data integrity")
        if split:
            fields = [split_correction(idx, [p[idx] for p in per_kernel]) for idx in range(ns)]
            potentials = [sum(f[i] for f in fields) for i in range(len(per_kernel))]
        else:
            potentials = [p.sum(dim=0) for p in per_kernel]
    else:
        for idx, field in enumerate(src_func):
            field_pot, _ = wrangler.eval_direct(
                traversal.target_boxes, traversal.neighbor_source_boxes_starts,
                traversal.neighbor_source_boxes_lists, field)
            if _contains_nonfinite(field_pot):
                raise RuntimeError(
                    "table-based list1 evaluation produced non-finite values for "
                    f"field {idx}; check near-field table data integrity")
            if split:
                field_pot = split_correction(idx, field_pot)
            potentials = field_pot if potentials is None else _add(potentials, field_pot)

    result = potentials
    if reorder_potentials:
        result = wrangler.reorder_potentials(potentials)
    result = wrangler.finalize_potentials(result)
    logger.info("fmm complete with list 1 only")
    return result
