"""Three-sequence alignment: ``Sequence.Align.align_3_powell`` and its
external ``powell_3d`` (src/sequence.ml:1309-1321; powell_3D_align,
src/ukkCommon.c:109-150, src/ukk.checkp.c) over the C ABI's
``poyalgn_powell_3d`` and ``poyalgn_powell_3d_batch``.

The GPU runs many triples per launch, one thread per triple replaying the
reference's check-pointed Ukkonen recursion; results are identical to the
reference's. There is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check
from .align import Context, CostMatrix

_P = C.c_void_p


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def powell_costs(cm: CostMatrix) -> tuple[int, int, int]:
    """(mm, go, ge) as align_3_powell_inter derives them from a 2D cost
    matrix (src/sequence.ml:1323-1337): the A/C cost, the affine gap opening
    (0 for linear and no-alignment models) and the A/gap cost."""
    t = cm.tables()
    cost = t["cost"]
    lcm = t["lcm"]
    mm = int(cost[(1 << lcm) + 2])
    ge = int(cost[(1 << lcm) + 16])
    go = int(t["gap_open"]) if t["cost_model"] == 1 else 0
    return mm, go, ge


def align_3_powell(ctx: Context, s1, s2, s3, mm: int, go: int, ge: int):
    """Sequence.Align.align_3_powell: the three aligned sequences (leading
    gap first) and the alignment cost."""
    a, b, c = (np.ascontiguousarray(x, np.uint8) for x in (s1, s2, s3))
    cap = len(a) + len(b) + len(c)
    ra, rb, rc = (np.zeros(cap, np.uint8) for _ in range(3))
    n, cost = C.c_int32(), C.c_int32()
    check(_lib.load().poyalgn_powell_3d(ctx.handle, _ptr(a), len(a), _ptr(b), len(b), _ptr(c),
                                        len(c), int(mm), int(go), int(ge), _ptr(ra), _ptr(rb),
                                        _ptr(rc), cap, C.byref(n), C.byref(cost)))
    k = n.value
    return ra[cap - k:].copy(), rb[cap - k:].copy(), rc[cap - k:].copy(), cost.value


@dataclass
class Powell3DBatch:
    cost: np.ndarray      # per triple (-1 where status is not 0)
    rlen: np.ndarray      # aligned length, leading gap included
    status: np.ndarray    # POYALGN_PAIR_* per triple
    out_off: np.ndarray   # triple k's alignments end at out_off[k] + cap[k]
    cap: np.ndarray
    ra: np.ndarray
    rb: np.ndarray
    rc: np.ndarray
    kernel_ms: float      # summed kernel time of the batch
    rounds: int           # launch rounds (budget splits and window reruns)

    def aligned(self, k: int):
        e = int(self.out_off[k] + self.cap[k])
        n = int(self.rlen[k])
        return self.ra[e - n:e], self.rb[e - n:e], self.rc[e - n:e]


def pack_triples(triples):
    """Concatenate triples of POY sequences: (seqs, off[3n], len[3n],
    out_off[n], cap[n])."""
    lens = np.array([[len(x) for x in t] for t in triples], np.int32).reshape(-1)
    off = np.zeros(len(lens), np.int64)
    if len(lens):
        off[1:] = np.cumsum(lens[:-1], dtype=np.int64)
    seqs = (np.concatenate([np.asarray(x, np.uint8) for t in triples for x in t])
            if len(lens) else np.zeros(1, np.uint8))
    cap = lens.reshape(-1, 3).sum(axis=1).astype(np.int64) if len(lens) else np.zeros(0, np.int64)
    out_off = np.zeros(len(cap), np.int64)
    if len(cap):
        out_off[1:] = np.cumsum(cap[:-1])
    return np.ascontiguousarray(seqs), off, lens, out_off, cap


def powell_3d_batch(ctx: Context, triples, mm: int, go: int, ge: int,
                    budget_bytes: int | None = None, raise_on_error: bool = True) -> Powell3DBatch:
    """align_3_powell on many triples at once (poyalgn_powell_3d_batch).

    budget_bytes, when given, caps the device memory the triples' workspaces
    take at once for this and every later batch on ctx (0 restores the
    default: half the free memory, at most 192 GB)."""
    lib = _lib.load()
    if budget_bytes is not None:
        check(lib.poyalgn_powell_3d_set_budget(ctx.handle, int(budget_bytes)))
    seqs, off, lens, out_off, cap = pack_triples(triples)
    n = len(cap)
    tot = int(cap.sum()) if n else 1
    ra, rb, rc = (np.zeros(max(tot, 1), np.uint8) for _ in range(3))
    rlen, cost, status = (np.zeros(max(n, 1), np.int32) for _ in range(3))
    rcode = lib.poyalgn_powell_3d_batch(ctx.handle, n, _ptr(seqs), _ptr(off), _ptr(lens),
                                        int(mm), int(go), int(ge), _ptr(out_off), _ptr(ra),
                                        _ptr(rb), _ptr(rc), _ptr(rlen), _ptr(cost), _ptr(status))
    if rcode != 0 and (raise_on_error or rcode != _lib.EPAIR):
        check(rcode)
    ms, rounds = C.c_float(), C.c_int32()
    check(lib.poyalgn_powell_3d_stats(ctx.handle, C.byref(ms), C.byref(rounds)))
    return Powell3DBatch(cost[:n], rlen[:n], status[:n], out_off, cap, ra, rb, rc,
                         float(ms.value), int(rounds.value))
