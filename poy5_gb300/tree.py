"""Device-resident node sequences and the level-batched tree downpass.

``Store`` keeps leaves and computed medians on the GPU (``poyalgn_store_*``);
``downpass`` computes every internal node's DOS.median bottom-up, one batch
per tree level, as AllDirChar.internal_downpass (src/allDirChar.ml:1366)
does one node at a time.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .align import Context, CostMatrix, _ptr, _u8, check


class Store:
    def __init__(self, ctx: Context, capacity_bytes: int):
        self.ctx = ctx
        h = C.c_void_p()
        check(_lib.load().poyalgn_store_create(ctx.handle, int(capacity_bytes), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def add(self, seq) -> int:
        s = _u8(seq)
        node = C.c_int32()
        check(_lib.load().poyalgn_store_add(self._h, _ptr(s), len(s), C.byref(node)))
        return node.value

    def __len__(self) -> int:
        return _lib.load().poyalgn_store_count(self._h)

    def read(self, node: int) -> np.ndarray:
        n = _lib.load().poyalgn_store_length(self._h, node)
        if n < 0:
            check(n)
        out = np.zeros(n, np.uint8)
        check(_lib.load().poyalgn_store_read(self._h, node, _ptr(out), n))
        return out

    def truncate(self, nodes: int):
        check(_lib.load().poyalgn_store_truncate(self._h, nodes))

    def median_batch(self, cm: CostMatrix, node_a, node_b, keep: bool = True):
        """DOS.median of resident pairs; returns (median nodes, costs, maxcosts, status)."""
        na = np.ascontiguousarray(node_a, np.int32)
        nb = np.ascontiguousarray(node_b, np.int32)
        n = len(na)
        med = np.full(n, -1, np.int32)
        cost, mx, st = (np.zeros(n, np.int32) for _ in range(3))
        rc = _lib.load().poyalgn_store_median_batch(self._h, cm.handle, n, _ptr(na), _ptr(nb),
                                                    int(keep), _ptr(med), _ptr(cost), _ptr(mx),
                                                    _ptr(st))
        if rc not in (0, _lib.EPAIR):
            check(rc)
        return med, cost, mx, st

    def median3_batch(self, cm: CostMatrix, parent, child1, child2):
        """SeqCS.DOS.median_3_no_union of resident triples (parent state, two
        children); returns (new nodes, costs, maxcosts, status)."""
        p = np.ascontiguousarray(parent, np.int32)
        a = np.ascontiguousarray(child1, np.int32)
        b = np.ascontiguousarray(child2, np.int32)
        n = len(p)
        node = np.full(n, -1, np.int32)
        cost, mx, st = (np.zeros(n, np.int32) for _ in range(3))
        rc = _lib.load().poyalgn_store_median3_batch(self._h, cm.handle, n, _ptr(p), _ptr(a),
                                                     _ptr(b), _ptr(node), _ptr(cost), _ptr(mx),
                                                     _ptr(st))
        if rc not in (0, _lib.EPAIR):
            check(rc)
        return node, cost, mx, st

    def closest_batch(self, cm: CostMatrix, node1, node2):
        """Sequence.Align.closest of resident pairs: node2 resolved towards
        node1; returns (new nodes, costs, status)."""
        a = np.ascontiguousarray(node1, np.int32)
        b = np.ascontiguousarray(node2, np.int32)
        n = len(a)
        node = np.full(n, -1, np.int32)
        cost, st = np.zeros(n, np.int32), np.zeros(n, np.int32)
        rc = _lib.load().poyalgn_store_closest_batch(self._h, cm.handle, n, _ptr(a), _ptr(b),
                                                     _ptr(node), _ptr(cost), _ptr(st))
        if rc not in (0, _lib.EPAIR):
            check(rc)
        return node, cost, st

    def readjust_batch(self, cm: CostMatrix, child_a, child_b, parent):
        """Sequence.readjust of resident triples; returns (centre nodes,
        cost3, cost2, status). The intermediate medians stay in the store."""
        a = np.ascontiguousarray(child_a, np.int32)
        b = np.ascontiguousarray(child_b, np.int32)
        p = np.ascontiguousarray(parent, np.int32)
        n = len(a)
        node = np.full(n, -1, np.int32)
        c3, c2, st = (np.zeros(n, np.int32) for _ in range(3))
        rc = _lib.load().poyalgn_store_readjust_batch(self._h, cm.handle, n, _ptr(a), _ptr(b),
                                                      _ptr(p), _ptr(node), _ptr(c3), _ptr(c2),
                                                      _ptr(st))
        if rc not in (0, _lib.EPAIR):
            check(rc)
        return node, c3, c2, st

    def close(self):
        if self._h:
            _lib.load().poyalgn_store_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class DownpassResult:
    internal_node: np.ndarray   # store node of each internal node's median
    internal_cost: np.ndarray   # DOS.median cost at each internal node
    total_cost: int
    levels: int


def downpass(store: Store, cm: CostMatrix, leaf_nodes, left, right) -> DownpassResult:
    """Median and cost of every internal node; see poyalgn_downpass."""
    leaf = np.ascontiguousarray(leaf_nodes, np.int32)
    lt = np.ascontiguousarray(left, np.int32)
    rt = np.ascontiguousarray(right, np.int32)
    ni = len(lt)
    node = np.full(ni, -1, np.int32)
    cost = np.zeros(ni, np.int32)
    total = C.c_int64()
    levels = C.c_int32()
    check(_lib.load().poyalgn_downpass(store.handle, cm.handle, len(leaf), _ptr(leaf), ni,
                                       _ptr(lt), _ptr(rt), _ptr(node), _ptr(cost),
                                       C.byref(total), C.byref(levels)))
    return DownpassResult(node, cost, int(total.value), int(levels.value))


@dataclass
class UppassResult:
    final_node: np.ndarray   # store node of each internal node's final state
    final_cost: np.ndarray   # cost2 of the alignment median_3 kept (0 at the root)
    levels: int


def uppass(store: Store, cm: CostMatrix, leaf_nodes, left, right, internal_node) -> UppassResult:
    """Final states top down from a downpass; see poyalgn_uppass."""
    leaf = np.ascontiguousarray(leaf_nodes, np.int32)
    lt = np.ascontiguousarray(left, np.int32)
    rt = np.ascontiguousarray(right, np.int32)
    inode = np.ascontiguousarray(internal_node, np.int32)
    ni = len(lt)
    node = np.full(ni, -1, np.int32)
    cost = np.zeros(ni, np.int32)
    levels = C.c_int32()
    check(_lib.load().poyalgn_uppass(store.handle, cm.handle, len(leaf), _ptr(leaf), ni,
                                     _ptr(lt), _ptr(rt), _ptr(inode), _ptr(node), _ptr(cost),
                                     C.byref(levels)))
    return UppassResult(node, cost, int(levels.value))


def tree_levels(nleaves: int, left, right) -> np.ndarray:
    """Level of each internal node (1 + the deeper child's; leaves are 0)."""
    lv = np.zeros(len(left), np.int32)
    for k, (a, b) in enumerate(zip(left, right)):
        for ch in (a, b):
            if not 0 <= ch < nleaves + k:
                raise ValueError(f"internal node {k}: child {ch} is not an earlier node")
        la = 0 if a < nleaves else lv[a - nleaves]
        lb = 0 if b < nleaves else lv[b - nleaves]
        lv[k] = 1 + max(la, lb)
    return lv
