"""Host-side mirror of POY's alignment interface over libpoyalgn.so.

Names and argument meaning follow the OCaml modules the CUDA library stands
in for (paths relative to the POY 5.1.1 source tree):

* :class:`CostMatrix` -- ``Cost_matrix.Two_D`` construction
  (``of_transformations_and_gaps``, ``of_list``, ``set_cost_model``),
  src/cost_matrix.ml:1003-1017, 1140-1189, 1300-1348.
* :class:`Align` -- ``Sequence.Align`` (src/sequence.ml:596-1826): ``cost_2``,
  ``create_edited_2``, ``align_2``, ``align_affine_3``, ``ancestor_2``,
  ``max_cost_2``; plus ``Sequence.median_2_with_gaps`` (:473-481).
* :func:`dos_median` -- ``SeqCS.DOS.median`` (src/seqCS.ml:985-1084), and
  :func:`median_batch`, the same for many pairs in one launch sequence.

Sequences are ``numpy.uint8`` arrays of POY bitset states (A=1 C=2 G=4 T=8,
gap=16) starting with the leading gap. Errors POY raises with ``failwith``
raise :class:`PoyAlgnError` here.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import PoyAlgnError, check

GAP = 16
_P = C.c_void_p


def _u8(s) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(s, dtype=np.uint8))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def encode(text: str) -> np.ndarray:
    """IUPAC DNA text to a bitset sequence with the leading gap."""
    code = {"A": 1, "C": 2, "G": 4, "T": 8, "-": 16, "R": 5, "Y": 10, "S": 6,
            "W": 9, "K": 12, "M": 3, "B": 14, "D": 13, "H": 11, "V": 7, "N": 15}
    return np.array([GAP] + [code[c] for c in text.upper()], np.uint8)


class Context:
    """A device binding (poyalgn_init). Not reentrant, like Matrix.default."""

    def __init__(self, device: int = 0):
        lib = _lib.load()
        h = _P()
        check(lib.poyalgn_init(device, C.byref(h)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            _lib.load().poyalgn_free(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_launches(self) -> int:
        return _lib.load().poyalgn_last_launches(self._h)

    def set_row_tile(self, mode: int):
        """0: lane pipeline, 1: row tile, 2: by batch size (lean affine passes)."""
        check(_lib.load().poyalgn_set_row_tile(self._h, int(mode)))

    def set_speculation(self, mode: int, passes: int = 8):
        """Speculative band passes: 0 off, 1 every batch, 2 by batch size
        (default); `passes` bands of each pair run at once."""
        check(_lib.load().poyalgn_set_speculation(self._h, int(mode), int(passes)))

    def set_memory_budget(self, slab_bytes: int = 0, arena_bytes: int = 0):
        """Cap the direction slabs and the deferred-traceback arena (0: default)."""
        check(_lib.load().poyalgn_set_memory_budget(self._h, int(slab_bytes), int(arena_bytes)))

    def profile_begin(self, max_batches: int):
        """Record per-launch CUDA events for the next `max_batches` batches."""
        check(_lib.load().poyalgn_profile_begin(self._h, int(max_batches)))

    def profile_end(self) -> dict:
        """Summed ms per launch slot: {'prep': t, 'class0': t, ...}."""
        lib = _lib.load()
        n = lib.poyalgn_num_classes()
        ms = np.zeros(n + 1, np.float32)
        nb = C.c_int()
        check(lib.poyalgn_profile_end(self._h, _ptr(ms), C.byref(nb)))
        out = {"prep": float(ms[0]), "batches": nb.value}
        for k in range(n):
            out[f"class{k}"] = float(ms[k + 1])
        return out


class CostMatrix:
    """Device-resident cost tables of a bitset alphabet (POY ``struct cm``)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self._h = handle
        t = self.tables()
        self.lcm, self.gap, self.a_sz = t["lcm"], t["gap"], t["a_sz"]
        self.cost_model, self.gap_open = t["cost_model"], t["gap_open"]

    @property
    def handle(self):
        return self._h

    @property
    def affine(self) -> bool:
        return self.cost_model == 1

    @classmethod
    def of_list(cls, ctx: Context, tcm, gap_open: int = 0) -> "CostMatrix":
        """fill_cost_matrix on a square matrix (gap last), then Affine go."""
        m = np.ascontiguousarray(np.asarray(tcm, dtype=np.int32))
        if m.ndim != 2 or m.shape[0] != m.shape[1]:
            raise ValueError("transformation cost matrix must be square")
        h = _P()
        check(_lib.load().poyalgn_cm_build(ctx.handle, _ptr(m), m.shape[0],
                                           int(gap_open), C.byref(h)))
        return cls(ctx, h)

    @classmethod
    def of_transformations_and_gaps(cls, ctx: Context, subs: int = 1,
                                    indel: int = 2, gap_open: int = 0,
                                    alph: int = 5) -> "CostMatrix":
        """POY's default DNA matrix: 0 diagonal, ``indel`` to the gap,
        ``subs`` elsewhere (src/cost_matrix.ml:1337-1348)."""
        tcm = [[0 if r == c else (indel if (r == alph - 1 or c == alph - 1) else subs)
                for c in range(alph)] for r in range(alph)]
        return cls.of_list(ctx, tcm, gap_open)

    @classmethod
    def adopt(cls, ctx: Context, lcm, gap, a_sz, combinations, cost_model,
              gap_open, cost, median, worst, tail, prepend) -> "CostMatrix":
        """Take the five tables of an existing POY ``struct cm``."""
        arrs = [np.ascontiguousarray(np.asarray(x, dtype=dt)) for x, dt in
                ((cost, np.int32), (median, np.uint8), (worst, np.int32),
                 (tail, np.int32), (prepend, np.int32))]
        h = _P()
        check(_lib.load().poyalgn_cm_adopt(ctx.handle, lcm, gap, a_sz, combinations,
                                           cost_model, gap_open,
                                           *(_ptr(a) for a in arrs), C.byref(h)))
        return cls(ctx, h)

    def tables(self) -> dict:
        n = 8192
        cost, worst, tail, prep = (np.zeros(n, np.int32) for _ in range(4))
        med = np.zeros(n, np.uint8)
        info = np.zeros(7, np.int32)
        k = _lib.load().poyalgn_cm_tables(self._h, _ptr(cost), _ptr(med), _ptr(worst),
                                          _ptr(tail), _ptr(prep), _ptr(info))
        return dict(cost=cost[:k], median=med[:k], worst=worst[:k], tail=tail[:k],
                    prepend=prep[:k], lcm=int(info[0]), gap=int(info[1]),
                    a_sz=int(info[2]), combinations=int(info[3]),
                    cost_model=int(info[4]), gap_open=int(info[5]),
                    min_non0_cost=int(info[6]))

    def close(self):
        if self._h:
            _lib.load().poyalgn_cm_free(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def count_gaps(s: np.ndarray, gap: int = GAP) -> int:
    """Sequence.Align.count_gaps (seq_CAML_count with startNO = 0)."""
    s = np.asarray(s)
    return int(np.count_nonzero((s >= gap) & ((s & gap) != 0)))


def deltaw_calc(s1len: int, s2len: int, deltaw: int | None = None) -> int:
    """The local ``deltaw_calc`` of Sequence.Align.cost_2 (src/sequence.ml:872-881)."""
    dif = s1len - s2len
    lower = int(float(s1len) * 0.10)
    if deltaw is None:
        return lower // 2 if dif < lower else 2
    return lower if dif < lower else deltaw


class Align:
    """Sequence.Align over one context (src/sequence.ml:596-1826)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.lib = _lib.load()

    # -- linear ---------------------------------------------------------
    def c_cost_2(self, s1, s2, cm: CostMatrix, deltawh: int) -> int:
        """The ``c_cost_2`` external: algn_CAML_simple_2 (s1 shorter)."""
        s1, s2 = _u8(s1), _u8(s2)
        out = C.c_int32()
        check(self.lib.poyalgn_simple_2(self.ctx.handle, cm.handle, _ptr(s1), len(s1),
                                        _ptr(s2), len(s2), int(deltawh), C.byref(out)))
        return out.value

    def cost_2(self, s1, s2, cm: CostMatrix, deltaw: int | None = None) -> int:
        """Linear cost with the facade's ordering and band seed."""
        if cm.affine:
            raise NotImplementedError("cost-only affine alignment (cost_2_affine) "
                                      "is not in the GPU library yet")
        s1, s2 = _u8(s1), _u8(s2)
        gaps = max(count_gaps(s1, cm.gap), count_gaps(s2, cm.gap))
        if len(s1) <= len(s2):
            return self.c_cost_2(s1, s2, cm, gaps + deltaw_calc(len(s1), len(s2), deltaw))
        return self.c_cost_2(s2, s1, cm, gaps + deltaw_calc(len(s2), len(s1), deltaw))

    def extract_edited_2(self, s1, s2, cm: CostMatrix, swap: int):
        """algn_CAML_backtrace_2d on the last c_cost_2 fill."""
        s1, s2 = _u8(s1), _u8(s2)
        cap = len(s1) + len(s2)
        p1, p2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
        n = C.c_int32()
        check(self.lib.poyalgn_backtrace_2d(self.ctx.handle, cm.handle, _ptr(s1), len(s1),
                                            _ptr(s2), len(s2), _ptr(p1), _ptr(p2), cap,
                                            C.byref(n), int(swap)))
        return p1[cap - n.value:], p2[cap - n.value:]

    def create_edited_2(self, s1, s2, cm: CostMatrix):
        """Aligned pair in caller order after cost_2 (src/sequence.ml:1019-1033)."""
        s1, s2 = _u8(s1), _u8(s2)
        if len(s1) <= len(s2):
            return self.extract_edited_2(s1, s2, cm, 0)
        p2, p1 = self.extract_edited_2(s2, s1, cm, 1)
        return p1, p2

    def limit_2(self, s1, s2, cm: CostMatrix, w: int, h: int, s1_st: int, s2_st: int,
                s1_len: int, s2_len: int) -> int:
        """The ``c_cost_2_limit`` external: algn_CAML_limit_2 (s1 shorter)."""
        s1, s2 = _u8(s1), _u8(s2)
        out = C.c_int32()
        check(self.lib.poyalgn_limit_2(self.ctx.handle, cm.handle, _ptr(s1), len(s1),
                                       _ptr(s2), len(s2), int(w), int(h), int(s1_st),
                                       int(s2_st), int(s1_len), int(s2_len), C.byref(out)))
        return out.value

    def backtrace_2d_limit(self, s1, s2, cm: CostMatrix, st_s1: int, st_s2: int,
                           algn_s1: int, algn_s2: int, swap: int):
        """The ``extract_edited_2_limit`` external on the last fill."""
        s1, s2 = _u8(s1), _u8(s2)
        cap = len(s1) + len(s2)
        p1, p2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
        n = C.c_int32()
        check(self.lib.poyalgn_backtrace_2d_limit(
            self.ctx.handle, cm.handle, _ptr(s1), len(s1), _ptr(s2), len(s2), _ptr(p1),
            _ptr(p2), cap, C.byref(n), int(st_s1), int(st_s2), int(algn_s1), int(algn_s2),
            int(swap)))
        return p1[cap - n.value:], p2[cap - n.value:]

    def verify_2(self, a, b, cm: CostMatrix) -> int:
        """algn_CAML_verify_2: cost of an aligned pair under cm's cost table."""
        a, b = _u8(a), _u8(b)
        out = C.c_int32()
        check(self.lib.poyalgn_verify_2(self.ctx.handle, cm.handle, _ptr(a), _ptr(b), len(a),
                                        C.byref(out)))
        return out.value

    def median_2_no_gaps(self, a, b, cm: CostMatrix) -> np.ndarray:
        """seq_CAML_median_2_no_gaps: the non-gap column medians after a gap."""
        a, b = _u8(a), _u8(b)
        cap = len(a) + 1
        out = np.zeros(cap, np.uint8)
        n = C.c_int32()
        check(self.lib.poyalgn_median_2_no_gaps(self.ctx.handle, cm.handle, _ptr(a), _ptr(b),
                                                len(a), _ptr(out), cap, C.byref(n)))
        return out[cap - n.value:]

    # -- affine ----------------------------------------------------------
    def c_align_affine_3(self, si, sj, cm: CostMatrix, swaped: int):
        si, sj = _u8(si), _u8(sj)
        cap = len(si) + len(sj) + 2
        bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
        lens = np.zeros(3, np.int32)
        cost = C.c_int32()
        check(self.lib.poyalgn_align_affine_3(self.ctx.handle, cm.handle, _ptr(si), len(si),
                                              _ptr(sj), len(sj), *(_ptr(b) for b in bufs),
                                              cap, _ptr(lens), int(swaped), C.byref(cost)))
        L, ml, wl = (int(x) for x in lens)
        return (bufs[0][cap - L:], bufs[1][cap - L:], bufs[2][cap - ml:],
                bufs[3][cap - wl:], cost.value)

    def align_affine_3(self, si, sj, cm: CostMatrix):
        """(median, aligned si, aligned sj, cost, median with gaps), caller order."""
        si, sj = _u8(si), _u8(sj)
        if len(si) <= len(sj):
            ri, rj, med, mwg, cost = self.c_align_affine_3(si, sj, cm, 0)
            return med, ri, rj, cost, mwg
        ri, rj, med, mwg, cost = self.c_align_affine_3(sj, si, cm, 1)
        return med, rj, ri, cost, mwg

    # -- both ------------------------------------------------------------
    def align_2(self, s1, s2, cm: CostMatrix):
        """(s1p, s2p, cost) with the leading gaps (src/sequence.ml:1061-1082)."""
        if cm.affine:
            _, p1, p2, cost, _ = self.align_affine_3(s1, s2, cm)
            return p1, p2, cost
        cost = self.cost_2(s1, s2, cm)
        p1, p2 = self.create_edited_2(s1, s2, cm)
        return p1, p2, cost

    def _aligned(self, a, b, cm: CostMatrix):
        a, b = _u8(a), _u8(b)
        if len(a) != len(b):
            raise ValueError("The size of the sequences is not the same.")
        cap = len(a) + 1
        anc = np.zeros(cap, np.uint8)
        mwg = np.zeros(len(a), np.uint8)
        alen, worst = C.c_int32(), C.c_int32()
        check(self.lib.poyalgn_aligned_medians(self.ctx.handle, cm.handle, _ptr(a), _ptr(b),
                                               len(a), _ptr(anc), cap, C.byref(alen),
                                               _ptr(mwg), C.byref(worst)))
        return anc[cap - alen.value:], mwg, worst.value

    def ancestor_2(self, a, b, cm: CostMatrix) -> np.ndarray:
        return self._aligned(a, b, cm)[0]

    def median_2_with_gaps(self, a, b, cm: CostMatrix) -> np.ndarray:
        return self._aligned(a, b, cm)[1]

    def cost_affine_3(self, si, sj, cm: CostMatrix) -> int:
        """algn_CAML_cost_affine_3: full unbanded affine cost, no traceback."""
        si, sj = _u8(si), _u8(sj)
        c = C.c_int32()
        check(_lib.load().poyalgn_cost_affine_3(self.ctx.handle, cm.handle, _ptr(si), len(si),
                                                _ptr(sj), len(sj), C.byref(c)))
        return c.value

    def max_cost_2(self, a, b, cm: CostMatrix) -> int:
        a, b = _u8(a), _u8(b)
        if np.all(a == cm.gap) or np.all(b == cm.gap):
            return 0
        return self._aligned(a, b, cm)[2]


@dataclass
class DOSMedian:
    """What SeqCS.DOS.median computes for one pair (Algn_Normal)."""
    median: np.ndarray      # seqm: ancestor (linear) / backtrace median (affine)
    aligned_a: np.ndarray   # tmpa
    aligned_b: np.ndarray   # tmpb
    cost: int               # tmpcost
    median_wg: np.ndarray   # seqmwg
    maxcost: int


def dos_median(align: Align, a, b, cm: CostMatrix) -> DOSMedian:
    """One SeqCS.DOS.median through the per-call entry points."""
    a, b = _u8(a), _u8(b)
    if cm.affine:
        med, pa, pb, cost, mwg = align.align_affine_3(a, b, cm)
        return DOSMedian(med, pa, pb, cost, mwg, align.max_cost_2(pa, pb, cm))
    pa, pb, cost = align.align_2(a, b, cm)
    anc, mwg, worst = align._aligned(pa, pb, cm)
    maxcost = 0 if (np.all(pa == cm.gap) or np.all(pb == cm.gap)) else worst
    return DOSMedian(anc, pa, pb, cost, mwg, maxcost)


@dataclass
class BatchResult:
    cost: np.ndarray
    maxcost: np.ndarray
    status: np.ndarray
    passes: np.ndarray
    alen: np.ndarray
    mlen: np.ndarray
    wlen: np.ndarray
    out_off: np.ndarray
    cap: np.ndarray
    ea: np.ndarray
    eb: np.ndarray
    med: np.ndarray
    mwg: np.ndarray

    def __len__(self):
        return len(self.cost)

    def _get(self, buf, k, n):
        end = int(self.out_off[k] + self.cap[k])
        return buf[end - int(n):end]

    def pair(self, k: int) -> DOSMedian:
        return DOSMedian(self._get(self.med, k, self.mlen[k]),
                         self._get(self.ea, k, self.alen[k]),
                         self._get(self.eb, k, self.alen[k]), int(self.cost[k]),
                         self._get(self.mwg, k, self.wlen[k]), int(self.maxcost[k]))


@dataclass
class PackedPairs:
    """A batch of pairs laid out for the batched entry points."""
    seqs: np.ndarray
    offa: np.ndarray
    lena: np.ndarray
    offb: np.ndarray
    lenb: np.ndarray
    out_off: np.ndarray
    cap: np.ndarray

    @property
    def npairs(self) -> int:
        return len(self.lena)

    @property
    def out_bytes(self) -> int:
        return int(self.out_off[-1] + self.cap[-1]) if len(self.cap) else 0

    @property
    def max_pair_len(self) -> int:
        return int((self.lena + self.lenb).max()) if len(self.lena) else 2


def pack_pairs(pairs) -> PackedPairs:
    """Concatenate (a, b) pairs and compute input/output offsets."""
    a_list = [_u8(a) for a, _ in pairs]
    b_list = [_u8(b) for _, b in pairs]
    lena = np.array([len(x) for x in a_list], np.int32)
    lenb = np.array([len(x) for x in b_list], np.int32)
    inter = [x for ab in zip(a_list, b_list) for x in ab]
    seqs = np.concatenate(inter) if inter else np.zeros(0, np.uint8)
    plen = (lena.astype(np.int64) + lenb)
    offa = np.zeros(len(lena), np.int64)
    if len(lena) > 1:
        offa[1:] = np.cumsum(plen)[:-1]
    offb = offa + lena
    cap = plen + 2
    out_off = np.zeros(len(lena), np.int64)
    if len(lena) > 1:
        out_off[1:] = np.cumsum(cap)[:-1]
    return PackedPairs(seqs, offa, lena, offb, lenb, out_off, cap)


def distance_batch(ctx: Context, cm: CostMatrix, pairs, missing_distance: int = 0):
    """SeqCS.DOS.distance of many pairs; returns (cost, status) arrays."""
    pk = pairs if isinstance(pairs, PackedPairs) else pack_pairs(pairs)
    n = pk.npairs
    cost = np.zeros(n, np.int32)
    status = np.zeros(n, np.int32)
    rc = _lib.load().poyalgn_distance_batch(
        ctx.handle, cm.handle, n, _ptr(pk.seqs), _ptr(pk.offa), _ptr(pk.lena), _ptr(pk.offb),
        _ptr(pk.lenb), int(missing_distance), _ptr(cost), _ptr(status))
    if rc not in (0, _lib.EPAIR):
        check(rc)
    return cost, status


def median_batch(ctx: Context, cm: CostMatrix, pairs) -> BatchResult:
    """DOS.median of many pairs through poyalgn_median_batch (host buffers)."""
    pk = pairs if isinstance(pairs, PackedPairs) else pack_pairs(pairs)
    n = pk.npairs
    tot = pk.out_bytes
    ints = [np.zeros(n, np.int32) for _ in range(7)]
    bufs = [np.zeros(max(tot, 1), np.uint8) for _ in range(4)]
    rc = _lib.load().poyalgn_median_batch(
        ctx.handle, cm.handle, n, _ptr(pk.seqs), _ptr(pk.offa), _ptr(pk.lena),
        _ptr(pk.offb), _ptr(pk.lenb), _ptr(pk.out_off), *(_ptr(x) for x in ints[:6]),
        *(_ptr(b) for b in bufs), _ptr(ints[6]))
    if rc not in (0, _lib.EPAIR):
        check(rc)
    return BatchResult(cost=ints[0], maxcost=ints[1], alen=ints[2], mlen=ints[3],
                       wlen=ints[4], status=ints[5], passes=ints[6], out_off=pk.out_off,
                       cap=pk.cap, ea=bufs[0], eb=bufs[1], med=bufs[2], mwg=bufs[3])
