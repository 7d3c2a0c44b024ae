"""``Sequence.NewkkAlign`` (src/sequence.ml:1831-1901) over libpoyalgn.so.

POY's own banded aligner (src/newkkonen.c) that ``SeqCS.DOS.median`` uses
when ``use_ukk`` is set. Only the affine cost model is provided: the
reference's linear variant leaves a zero-cost diagonal candidate in every
inner cell and its backtrace fails an assertion (src/newkkonen.c:796,
1554).

* :class:`NewkkAlign` -- ``align_2`` (shorter sequence first, ``swaped``)
  through the per-call stubs ``newkkonen_CAML_algn_affine`` and
  ``newkkonen_CAML_backtrace_affine``, and ``get_k``.
* :func:`newkk_median_batch` -- ``DOS.median`` with ``use_ukk`` for many
  pairs (align_2, then ``ancestor_2``, ``median_2_with_gaps`` and
  ``max_cost_2``), in the same result layout as :func:`median_batch`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import PoyAlgnError, check
from .align import BatchResult, Context, CostMatrix, PackedPairs, pack_pairs

_I = C.c_int32


def _u8(s) -> np.ndarray:
    return np.ascontiguousarray(s, dtype=np.uint8)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class NewkkAlign:
    """Sequence.NewkkAlign on one context (its ukkm matrix is the context)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def cost2_affine(self, s1, s2, cm: CostMatrix, swaped: int) -> int:
        """newkk_cost2_affine: s1 must be the shorter (failwith otherwise)."""
        s1, s2 = _u8(s1), _u8(s2)
        c = _I()
        check(_lib.load().poyalgn_newkk_algn_affine(
            self.ctx.handle, cm.handle, _ptr(s1), len(s1), _ptr(s2), len(s2),
            int(swaped), C.byref(c)))
        return c.value

    def backtrace_affine(self, s1, s2, cm: CostMatrix, swaped: int):
        """newkk_backtrace_affine of the last cost2_affine on (s1, s2)."""
        s1, s2 = _u8(s1), _u8(s2)
        cap = len(s1) + len(s2)
        p1 = np.zeros(cap, np.uint8)
        p2 = np.zeros(cap, np.uint8)
        n = _I()
        check(_lib.load().poyalgn_newkk_backtrace_affine(
            self.ctx.handle, cm.handle, _ptr(s1), len(s1), _ptr(s2), len(s2),
            _ptr(p1), _ptr(p2), cap, C.byref(n), int(swaped)))
        return p1[cap - n.value:].copy(), p2[cap - n.value:].copy()

    def set_arena_words(self, words: int):
        """Bound the direction-code arena (0: sized from free memory)."""
        check(_lib.load().poyalgn_newkk_set_arena_words(self.ctx.handle, int(words)))

    def get_k(self) -> int:
        k = _I()
        check(_lib.load().poyalgn_newkk_get_k(self.ctx.handle, C.byref(k)))
        return k.value

    def align_2(self, s1, s2, cm: CostMatrix):
        """align_2 ~first_gap:true: (aligned s1, aligned s2, cost) in the
        caller's order; the shorter sequence goes first (swaped = 1 when s2
        is the shorter), src/sequence.ml:1879-1901."""
        s1, s2 = _u8(s1), _u8(s2)
        if not cm.affine:
            raise PoyAlgnError(_lib.EUNSUPPORTED,
                               "Algn_Newkk is built for the affine cost model only")
        exchange = len(s1) > len(s2)
        a, b = (s2, s1) if exchange else (s1, s2)
        sw = 1 if exchange else 0
        cost = self.cost2_affine(a, b, cm, sw)
        pa, pb = self.backtrace_affine(a, b, cm, sw)
        return (pb, pa, cost) if exchange else (pa, pb, cost)


def newkk_median_batch(ctx: Context, cm: CostMatrix, pairs) -> BatchResult:
    """DOS.median with use_ukk of many pairs (host buffers)."""
    pk = pairs if isinstance(pairs, PackedPairs) else pack_pairs(pairs)
    n = pk.npairs
    tot = pk.out_bytes
    ints = [np.zeros(n, np.int32) for _ in range(7)]
    bufs = [np.zeros(max(tot, 1), np.uint8) for _ in range(4)]
    rc = _lib.load().poyalgn_newkk_median_batch(
        ctx.handle, cm.handle, n, _ptr(pk.seqs), _ptr(pk.offa), _ptr(pk.lena),
        _ptr(pk.offb), _ptr(pk.lenb), _ptr(pk.out_off), *(_ptr(x) for x in ints[:6]),
        *(_ptr(b) for b in bufs), _ptr(ints[6]))
    if rc not in (0, _lib.EPAIR):
        check(rc)
    return BatchResult(cost=ints[0], maxcost=ints[1], alen=ints[2], mlen=ints[3],
                       wlen=ints[4], status=ints[5], passes=ints[6], out_off=pk.out_off,
                       cap=pk.cap, ea=bufs[0], eb=bufs[1], med=bufs[2], mwg=bufs[3])


def newkk_distance_batch(ctx: Context, cm: CostMatrix, pairs, missing_distance: int = 0):
    """SeqCS.DOS.distance with use_ukk under an affine model (src/seqCS.ml:
    701-705, 745-747): ``missing_distance`` when either sequence is empty
    (every position the gap, ``Sequence.is_empty``), otherwise
    ``NewkkAlign.cost_2`` (src/sequence.ml:1938-1975), the Newkk cost of the
    pair with the shorter sequence first. Returns an int32 array."""
    gap = 16
    pairs = [(_u8(a), _u8(b)) for a, b in pairs]
    out = np.full(len(pairs), missing_distance, np.int32)
    live = [k for k, (a, b) in enumerate(pairs)
            if not (np.all(a == gap) or np.all(b == gap))]
    if live:
        res = newkk_median_batch(ctx, cm, [pairs[k] for k in live])
        # the cost needs the fill only: statuses the traceback or the medians
        # set (capacity, zero median, off band) leave it valid
        bad = np.nonzero(~np.isin(res.status, (0, -2, -3, -13)))[0]
        if len(bad):
            raise PoyAlgnError(_lib.EPAIR, "pair %d failed with status %d"
                               % (live[int(bad[0])], int(res.status[bad[0]])))
        out[live] = res.cost
    return out
