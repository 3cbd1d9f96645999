"""Mixed-precision (tensor-core) list-1 evaluation: host side.

``eval_mixed`` runs ``vl1_eval_mixed`` (``include/vl1.h``): the list-1 sum of
``volumential/list1.py:1050-1159`` computed from exact FP16 digit products on
the tcgen05 tensor cores with FP64 final sums (relative error ~2^-40 of
sum |table| |density|, see ``csrc/vl1_mixed.cu``).

The device kernel walks a *schedule*: tiles of 128 rows, each row one
(target box, right-hand side) item, and for each tile the list of table keys
(table level, interaction case) its target boxes use.  The schedule depends
only on the tree, the plan and the rhs count, so it is built once (from the
per-pair keys that ``vl1_classify_pairs`` computes with the reference's FP64
case encoding) and cached.  Target boxes are grouped by their key signature
(the set of keys of their pairs) and packed greedily into tiles with small
key unions, so that little tensor-core work is spent on rows without a pair
of the current key (on the C2 octree, 75 % of the rows of a tile key carry a
pair, against 57 % when the signatures are only sorted).
"""

from __future__ import annotations

import collections
import ctypes as C
import threading

import numpy as np

from . import _lib

__all__ = ["MixedSchedule", "get_schedule", "eval_mixed", "DIGITS", "ROWS_PER_TILE"]

DIGITS = 5
ROWS_PER_TILE = 128

_cache: "collections.OrderedDict" = collections.OrderedDict()
_lock = threading.Lock()
_CACHE_MAX = 256


class MixedSchedule:
    """Device-resident schedule (and workspace) of one (plan, tree, nrhs).

    ``packing``: "device" builds the schedule on the GPU
    (``vl1_schedule_build_*``: boxes ordered by key signature, a few
    milliseconds even for large trees; the path of a first call on a new
    tree); "greedy" classifies on the GPU and packs the tiles on the host
    with ``pack_rows`` (about 13 % fewer tile keys on the C2 octree, at
    ~1 s of host time), for trees evaluated many times."""

    def __init__(self, plan, view, keep, nrhs, stream, max_keys_per_item=None, base=None,
                 workspace=True, packing="device"):
        import torch

        lib = _lib.lib()
        self.nrhs = int(nrhs)
        self._workspace = None
        self.packing = packing if base is None else base.packing
        # bytes of vl1_eval_mixed's workspace, allocated on first use
        # (schedules of a batch use the batch's buffer instead)
        self.workspace_bytes = int(lib.vl1_mixed_workspace_bytes(plan.handle, C.byref(view),
                                                                 self.nrhs))
        if self.workspace_bytes < 0:
            raise RuntimeError("vl1_mixed_workspace_bytes failed")
        if base is not None:
            # same plan, tree and nrhs: only the work items differ
            self._init_items(plan, base, max_keys_per_item)
            if workspace:
                _ = self.workspace
            return
        if packing == "device":
            self._build_on_device(plan, view, keep, stream)
        elif packing == "greedy":
            self._build_on_host(plan, view, keep, stream)
        else:
            raise ValueError(f"packing must be 'device' or 'greedy', got {packing!r}")
        self._init_items(plan, self, max_keys_per_item)
        if workspace:
            _ = self.workspace

    @property
    def workspace(self):
        """Device workspace of ``vl1_eval_mixed`` (allocated on first use)."""
        if self._workspace is None:
            import torch

            self._workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8,
                                          device="cuda")
        return self._workspace

    def _build_on_device(self, plan, view, keep, stream):
        import torch

        lib = _lib.lib()
        nnz = int(keep["lists"].numel())
        sizes = _lib.ScheduleSizes()
        b = C.c_void_p()
        st = lib.vl1_schedule_build_begin(plan.handle, C.byref(view), nnz, self.nrhs,
                                          C.byref(b), C.byref(sizes), C.c_void_p(stream))
        if st == _lib.VL1_E_LAYOUT:
            raise ValueError("the mixed-precision path requires distinct source mode ids in "
                             f"[0, {plan.nq}) inside every box: {_lib.last_error()}")
        if st == _lib.VL1_E_ARG and "same case" in _lib.last_error():
            raise RuntimeError(_lib.last_error())
        _lib.check(st, "vl1_schedule_build_begin")
        try:
            n_tiles, n_ent = int(sizes.n_tiles), int(sizes.n_entries)
            key_start = np.empty(n_tiles + 1, dtype=np.int32)
            _lib.check(lib.vl1_schedule_build_key_start(b, key_start.ctypes.data),
                       "vl1_schedule_build_key_start")
            dev = lambda n: torch.empty(max(n, 1), dtype=torch.int32, device="cuda")  # noqa
            self.tile_rows = dev(n_tiles * ROWS_PER_TILE)
            self.tile_key_start = dev(n_tiles + 1)
            self.key_ids = dev(n_ent)
            self.key_xrow = dev(max(n_ent, 1) * ROWS_PER_TILE)
            _lib.check(lib.vl1_schedule_build_fill(
                b, self.tile_rows.data_ptr(), self.tile_key_start.data_ptr(),
                self.key_ids.data_ptr(), self.key_xrow.data_ptr(), C.c_void_p(stream)),
                "vl1_schedule_build_fill")
        finally:
            lib.vl1_schedule_builder_destroy(b)
        self.n_tiles = n_tiles
        self.n_tile_keys = n_ent
        self.mean_keys_per_tile = n_ent / max(n_tiles, 1)
        self.key_start_np = key_start.astype(np.int64)

    def _build_on_host(self, plan, view, keep, stream):
        import torch

        lib = _lib.lib()
        n_tb = int(view.n_target_boxes)
        nnz = int(keep["lists"].numel())
        n_keys_total = plan.n_tables * plan.n_cases
        keys_dev = torch.empty(max(nnz, 1), dtype=torch.int32, device="cuda")
        _lib.check(lib.vl1_classify_pairs(plan.handle, C.byref(view), keys_dev.data_ptr(),
                                          C.c_void_p(stream)), "vl1_classify_pairs")
        plan.raise_on_status(stream)
        keys = keys_dev[:nnz].cpu().numpy().astype(np.int64)
        starts = keep["starts"].cpu().numpy().astype(np.int64)
        lists = keep["lists"].cpu().numpy().astype(np.int64)
        self._check_modes(keep, plan.nq)

        tile_rows, key_start, key_ids, xrow = self.tile_schedule(
            keys, starts, lists, n_tb, n_keys_total, self.nrhs)
        n_tiles = len(tile_rows)

        self.n_tiles = n_tiles
        self.n_tile_keys = int(len(key_ids))
        self.mean_keys_per_tile = self.n_tile_keys / max(n_tiles, 1)
        self.tile_rows = torch.from_numpy(tile_rows.ravel().astype(np.int32)).to("cuda")
        self.tile_key_start = torch.from_numpy(key_start.astype(np.int32)).to("cuda")
        self.key_ids = torch.from_numpy(key_ids.astype(np.int32) if len(key_ids)
                                        else np.zeros(1, np.int32)).to("cuda")
        self.key_xrow = torch.from_numpy(xrow.ravel() if len(key_ids)
                                         else np.zeros(ROWS_PER_TILE, np.int32)).to("cuda")
        self.key_start_np = np.asarray(key_start, dtype=np.int64)

    def _init_items(self, plan, base, max_keys_per_item):
        """Work items, split counters and partial-sum scratch for a cap; the
        tile arrays come from ``base`` (this schedule or one of the same plan,
        tree and nrhs)."""
        import torch

        for name in ("n_tiles", "n_tile_keys", "mean_keys_per_tile", "tile_rows",
                     "tile_key_start", "key_ids", "key_xrow", "key_start_np"):
            setattr(self, name, getattr(base, name))
        key_start = self.key_start_np
        n_tiles = self.n_tiles
        geo = plan.mixed_geometry()
        n_chunks = geo["np"] // geo["nch"]
        # the work list depends only on the tiles and the cap: computed once
        # per base schedule (further instances, e.g. a server's per-request
        # slots, only allocate their own scratch)
        if not hasattr(base, "_items_memo"):
            base._items_memo = {}
        memo = base._items_memo.get(max_keys_per_item)
        if memo is None:
            memo = self._work_items(np.asarray(key_start, dtype=np.int64), max_keys_per_item)
            base._items_memo[max_keys_per_item] = memo
        items, n_splits, n_slots = memo
        self.n_items = len(items)
        self.n_splits = n_splits
        self.max_keys_per_item = int(max(1, (items[:, 2] - items[:, 1]).max()
                                         if len(items) else 1))
        # host copy (vl1_batch_problem.host_items) and device copy of the items
        self.items_np = np.ascontiguousarray(items if len(items)
                                             else np.zeros((1, 8), np.int32))
        self.items = torch.from_numpy(self.items_np).to("cuda")
        # one counter per split tile and column chunk, spaced 16 apart
        self.split_counters = torch.zeros(max(1, n_splits * n_chunks * 16), dtype=torch.int32,
                                          device="cuda")
        self.split_partials = torch.zeros(max(16, n_slots * ROWS_PER_TILE * geo["np"] * 8),
                                          dtype=torch.uint8, device="cuda")
        s = _lib.MixedSchedule()
        s.n_tiles = n_tiles
        s.tile_rows = self.tile_rows.data_ptr()
        s.tile_key_start = self.tile_key_start.data_ptr()
        s.key_ids = self.key_ids.data_ptr()
        s.key_xrow = self.key_xrow.data_ptr()
        s.n_items = len(items)
        s.items = self.items.data_ptr()
        s.n_splits = n_splits
        s.n_slots = n_slots
        s.split_counters = self.split_counters.data_ptr()
        s.split_partials = self.split_partials.data_ptr()
        s.n_chunks = n_chunks
        self.n_chunks = n_chunks
        self.geometry = (geo["kc"], geo["nch"])
        self.c_struct = s

    @staticmethod
    def tile_schedule(keys, starts, lists, n_tb, n_keys_total, nrhs, order=None):
        """Tiles of 128 (target box, rhs) rows and their (tile, key) entries.

        Target boxes are packed into tiles by their key signatures (the set
        of (table level, case) keys of their list-1 pairs, ``pack_rows``) so
        that a tile's rows share keys; tiles are ordered by key count, longest
        first.  Returns ``tile_rows``
        [n_tiles, 128] (row j * nrhs + r, or -1), ``key_start`` [n_tiles + 1],
        ``key_ids`` [n_entries] and ``xrow`` [n_entries, 128] (density row
        S * nrhs + r of the row's list-1 source box S for that key, or -1).
        ``order``: the box order to use instead of ``pack_rows``'s.
        """
        nnz = len(keys)
        K = n_keys_total
        tb_of_pair = np.repeat(np.arange(n_tb, dtype=np.int64), np.diff(starts))
        # target boxes grouped by key signature (the set of keys of their
        # pairs) and packed into tiles so that each tile's key union stays
        # small (every key of a tile costs all 128 rows their tensor work)
        if order is not None:
            order = np.asarray(order, dtype=np.int64)
        elif n_tb:
            mask = np.zeros((n_tb, K), dtype=bool)
            mask[tb_of_pair, keys] = True
            order = MixedSchedule.pack_rows(mask, max(1, ROWS_PER_TILE // nrhs))
        else:
            order = np.zeros(0, dtype=np.int64)
        n_rows = n_tb * nrhs
        n_tiles = (n_rows + ROWS_PER_TILE - 1) // ROWS_PER_TILE
        tile_rows = np.full(n_tiles * ROWS_PER_TILE, -1, dtype=np.int64)
        tile_rows[:n_rows] = (order[:, None] * nrhs + np.arange(nrhs)[None, :]).ravel()
        pos = np.empty(n_tb, dtype=np.int64)      # rank of each box in the row order
        pos[order] = np.arange(n_tb, dtype=np.int64)

        # (box, key) pairs must be unique: one list-1 source box per case
        comb = tb_of_pair * K + keys
        if len(comb) > 1:
            cs = np.sort(comb)
            if np.any(cs[1:] == cs[:-1]):
                raise RuntimeError("a target box has two list-1 source boxes with the same case")

        # (tile, key) entries: every tile that holds a row of a pair's target box
        first_tile = (pos * nrhs) // ROWS_PER_TILE
        span = (pos * nrhs + nrhs - 1) // ROWS_PER_TILE - first_tile + 1
        sp = span[tb_of_pair]
        rep = np.repeat(np.arange(nnz, dtype=np.int64), sp)
        offs = np.arange(len(rep), dtype=np.int64) - np.repeat(np.cumsum(sp) - sp, sp)
        codes = np.unique((first_tile[tb_of_pair][rep] + offs) * K + keys[rep])
        ent_tile = codes // K
        ent_key = codes % K
        n_keys_per_tile = np.bincount(ent_tile, minlength=n_tiles)
        # longest tiles first (CTAs start in grid order)
        lpt = np.argsort(-n_keys_per_tile, kind="stable")
        inv_lpt = np.empty(n_tiles, dtype=np.int64)
        inv_lpt[lpt] = np.arange(n_tiles, dtype=np.int64)
        new_tile = inv_lpt[ent_tile]
        o2 = np.lexsort((ent_key, new_tile))
        inv_o2 = np.empty(len(codes), dtype=np.int64)
        inv_o2[o2] = np.arange(len(codes), dtype=np.int64)
        key_ids = ent_key[o2]
        key_start = np.concatenate([[0], np.cumsum(np.bincount(new_tile, minlength=n_tiles))])
        tile_rows = tile_rows.reshape(n_tiles, ROWS_PER_TILE)[lpt]

        # density row of every (entry, tile slot): source box * nrhs + rhs, or -1
        xrow = np.full((len(codes), ROWS_PER_TILE), -1, dtype=np.int32)
        base_pos = pos[tb_of_pair] * nrhs
        for r in range(nrhs):
            P = base_pos + r
            e = inv_o2[np.searchsorted(codes, (P // ROWS_PER_TILE) * K + keys)]
            xrow[e, P % ROWS_PER_TILE] = (lists * nrhs + r).astype(np.int32)
        return tile_rows, key_start, key_ids, xrow

    @staticmethod
    def pack_rows(mask, rows_per_tile):
        """Order of the target boxes (rows of the bool matrix ``mask`` [boxes,
        keys]) that packs them into tiles of ``rows_per_tile`` with few keys
        per tile.  Boxes with equal key sets (signatures) stay together; a
        tile is filled greedily, starting from the signature with the most
        boxes left and then taking, at each step, the signature that adds the
        fewest new keys per box it contributes (ties: more boxes, then the
        earlier signature); boxes keep their index order inside a signature.
        """
        n, K = mask.shape
        words = -(-K // 64)
        padded = np.zeros((n, words * 64), dtype=bool)
        padded[:, :K] = mask
        # one uint64 per 64 keys (little-endian bit order inside each word)
        packed = np.packbits(padded.reshape(n, words, 8, 8)[:, :, ::-1, ::-1]
                             .reshape(n, words * 64), axis=1, bitorder="big")
        packed = packed.reshape(n, words, 8).view(">u8").reshape(n, words).astype(np.uint64)
        sigs, inv = np.unique(packed, axis=0, return_inverse=True)
        inv = inv.ravel()
        members = np.argsort(inv, kind="stable")               # boxes by signature
        bounds = np.concatenate([[0], np.cumsum(np.bincount(inv, minlength=len(sigs)))])
        rem = np.diff(bounds).astype(np.int64)
        taken = np.zeros(len(sigs), dtype=np.int64)
        out = np.empty(n, dtype=np.int64)
        filled = 0
        while filled < n:
            tile_keys = np.zeros(words, dtype=np.uint64)
            space = rows_per_tile
            s_ = int(np.argmax(rem))
            while True:
                take = int(min(space, rem[s_]))
                b0 = bounds[s_] + taken[s_]
                out[filled:filled + take] = members[b0:b0 + take]
                filled += take
                taken[s_] += take
                rem[s_] -= take
                space -= take
                tile_keys |= sigs[s_]
                if space == 0 or filled == n:
                    break
                new = np.bitwise_count(sigs & ~tile_keys).sum(axis=1).astype(np.float64)
                avail = rem > 0
                per_row = new / np.maximum(np.minimum(rem, space), 1)
                per_row[~avail] = np.inf
                best = per_row.min()
                cand = np.flatnonzero(per_row == best)
                s_ = int(cand[np.argmax(rem[cand])])
        return out

    @staticmethod
    def _work_items(key_start, max_keys_per_item, n_sm=None):
        """Work items (one CTA each): whole tiles, and tiles with more than a
        cap of keys split into nearly equal key ranges, ordered longest first
        (CTAs start in grid order).  Without an explicit cap, the cap with the
        shortest modelled finish time is taken (``vl1_mixed_work_items``).
        Returns (items [n_items, 8] int32, n_splits, n_slots)."""
        key_start = np.ascontiguousarray(key_start, dtype=np.int32)
        n_tiles = len(key_start) - 1
        cap = 0 if max_keys_per_item is None else max(1, int(max_keys_per_item))
        if n_sm is None:
            n_sm = 1
            if cap == 0:
                import torch

                n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()) \
                    .multi_processor_count
        capacity = int(key_start[-1]) + n_tiles + 1
        out = np.zeros((capacity, 8), dtype=np.int32)
        n_items, n_splits, n_slots = C.c_int32(), C.c_int32(), C.c_int32()
        _lib.check(_lib.lib().vl1_mixed_work_items(
            key_start.ctypes.data, n_tiles, cap, int(n_sm), out.ctypes.data, capacity,
            C.byref(n_items), C.byref(n_splits), C.byref(n_slots)), "vl1_mixed_work_items")
        return out[:n_items.value].copy(), int(n_splits.value), int(n_slots.value)

    @staticmethod
    def _check_modes(keep, nq):
        """Source mode ids must be distinct inside a box (the mixed path places
        every source point at its mode's column)."""
        counts = keep["src_counts"].cpu().numpy().astype(np.int64)
        starts = keep["src_starts"].cpu().numpy().astype(np.int64)
        smode = keep["smode"].cpu().numpy()
        boxes = np.flatnonzero(counts > 0)
        if not len(boxes):
            return
        c = np.minimum(counts[boxes], nq)
        full = c == nq
        if np.any(full):
            idx = starts[boxes[full]][:, None] + np.arange(nq)[None, :]
            m = np.sort(smode[idx], axis=1)
            if not np.array_equal(m, np.broadcast_to(np.arange(nq), m.shape)):
                raise ValueError(
                    "the mixed-precision path requires every box's source mode ids to be "
                    f"a permutation of 0..{nq - 1}")
        for b, cnt in zip(boxes[~full], c[~full]):
            m = smode[starts[b]:starts[b] + cnt]
            if len(np.unique(m)) != len(m):
                raise ValueError("duplicate source mode ids inside a box")


def _tree_token(keep):
    return tuple((t.data_ptr(), t._version, tuple(t.shape)) for t in keep.values())


def get_schedule(plan, view, keep, nrhs, stream, max_keys_per_item=None, packing=None):
    """The cached schedule of (plan, tree, nrhs, cap), built on a miss.

    ``packing`` None takes whatever schedule is cached for the tree (a new one
    is built on the device); "device" or "greedy" asks for that packing and
    replaces the tree's schedules of the other packing."""
    geo = plan.mixed_geometry()
    key = (id(plan), _tree_token(keep), int(nrhs), (geo["kc"], geo["nch"]), max_keys_per_item)
    with _lock:
        hit = _cache.get(key)
        if hit is not None and (packing is None or hit[0].packing == packing):
            _cache.move_to_end(key)
            return hit[0]
    base = None
    with _lock:
        for k, v in _cache.items():
            # same plan, tree and nrhs (any tile shape and cap): its tile
            # arrays are shared, only the work items and split scratch differ
            if k[:3] == key[:3] and (packing is None or v[0].packing == packing):
                base = v[0]
                break
    sched = MixedSchedule(plan, view, keep, nrhs, stream, max_keys_per_item, base=base,
                          packing=packing or "device", workspace=False)
    with _lock:
        if packing is not None:
            for k in [k for k, v in _cache.items()
                      if k[:3] == key[:3] and v[0].packing != sched.packing]:
                del _cache[k]
        # keep the tree tensors alive with the schedule so the token stays unique
        _cache[key] = (sched, dict(keep), plan)
        while len(_cache) > _CACHE_MAX:
            _cache.popitem(last=False)
    return sched


def eval_mixed(plan, view, coefs, out, *, stream, nrhs, keep, max_keys_per_item=None):
    """Tensor-core evaluation of ``nrhs`` right-hand sides into ``out``.

    ``coefs``: CUDA float64 (or complex128) tensor with ``nrhs * N`` values;
    ``out``: CUDA tensor of the plain path's output dtype and size.
    ``max_keys_per_item``: split tiles with more keys over several CTAs
    (default: one SM's share of the work).
    """
    import torch

    n = int(view.n_particles)
    if coefs.is_complex():
        # y(re + i im) = y(re) + i y(im): two real evaluations in one launch
        c2 = torch.cat([coefs.real.reshape(nrhs, n), coefs.imag.reshape(nrhs, n)]).contiguous()
        tmp = torch.empty((2 * nrhs, n), dtype=torch.complex128 if plan.complex_table
                          else torch.float64, device="cuda")
        eval_mixed(plan, view, c2, tmp, stream=stream, nrhs=2 * nrhs, keep=keep,
                   max_keys_per_item=max_keys_per_item)
        res = tmp[:nrhs] + 1j * tmp[nrhs:]
        out.view(nrhs, n).copy_(res)
        return
    if coefs.dtype != torch.float64 or not coefs.is_contiguous():
        raise TypeError("mixed path coefficients must be a contiguous float64 tensor")
    sched = get_schedule(plan, view, keep, nrhs, stream, max_keys_per_item)
    lib = _lib.lib()
    st = lib.vl1_eval_mixed(plan.handle, C.byref(view), C.byref(sched.c_struct),
                            coefs.data_ptr(), int(nrhs), out.data_ptr(),
                            sched.workspace.data_ptr(), int(sched.workspace.numel()),
                            C.c_void_p(stream))
    _lib.check(st, "vl1_eval_mixed")
