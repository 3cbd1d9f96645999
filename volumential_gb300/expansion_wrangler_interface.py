"""Expansion wrangler interface (``volumential/expansion_wrangler_interface.py``).

Kept for drop-in compatibility: ``drive_volume_fmm`` accepts any object with
these methods.  As in the reference, subclasses need not implement every
method (the reference's ``ABCMeta`` is inert under Python 3).
"""

from __future__ import annotations

__all__ = ["ExpansionWranglerInterface", "TreeIndependentDataForWranglerInterface"]


class ExpansionWranglerInterface:
    """Abstract expansion handling interface (boxtree/fmm compatible)."""

    def multipole_expansion_zeros(self):
        raise NotImplementedError

    def local_expansion_zeros(self):
        raise NotImplementedError

    def output_zeros(self):
        raise NotImplementedError

    def reorder_sources(self, source_array):
        raise NotImplementedError

    def reorder_targets(self, target_array):
        raise NotImplementedError

    def reorder_potentials(self, potentials):
        raise NotImplementedError

    def form_multipoles(self, level_start_source_box_nrs, source_boxes, src_weights):
        raise NotImplementedError

    def coarsen_multipoles(self, level_start_source_parent_box_nrs, source_parent_boxes,
                           mpoles):
        raise NotImplementedError

    def eval_direct(self, target_boxes, neighbor_sources_starts, neighbor_sources_lists,
                    mode_coefs):
        raise NotImplementedError

    def multipole_to_local(self, level_start_target_or_target_parent_box_nrs,
                           target_or_target_parent_boxes, starts, lists, mpole_exps):
        raise NotImplementedError

    def eval_multipoles(self, level_start_target_box_nrs, target_boxes, starts, lists,
                        mpole_exps):
        raise NotImplementedError

    def form_locals(self, level_start_target_or_target_parent_box_nrs,
                    target_or_target_parent_boxes, starts, lists, src_weights):
        raise NotImplementedError

    def refine_locals(self, level_start_target_or_target_parent_box_nrs,
                      target_or_target_parent_boxes, local_exps):
        raise NotImplementedError

    def eval_locals(self, level_start_target_box_nrs, target_boxes, local_exps):
        raise NotImplementedError

    def finalize_potentials(self, potentials):
        raise NotImplementedError


class TreeIndependentDataForWranglerInterface:
    def get_wrangler(self, *args, **kwargs):
        raise NotImplementedError
