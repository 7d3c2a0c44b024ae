"""Pipeline ladders and the autotuner.

A ladder is the list of (P lanes, R rows per lane) pipeline shapes a context
picks from as a pair's band doubles (class c takes bands up to
2 (P - 1) R + 1 wide). ``autotune`` times candidate ladders on a sample batch
through ``poyalgn_autotune`` (which also checks that every candidate gives
the same per-pair results) and keeps the fastest on the context.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .align import Context, CostMatrix, PackedPairs, _ptr, check, pack_pairs

NCLASS = 12
P_ALLOWED = (4, 8, 16, 32, 64, 128, 256, 512)


def default_ladder(affine: bool):
    if affine:
        return ([8, 8, 16, 16, 32, 32, 32, 64, 64, 128, 256, 512],
                [2, 3, 2, 3, 2, 3, 4, 3, 4, 4, 4, 4])
    return ([4, 8, 16, 32, 32, 32, 64, 128, 256, 512, 512, 512],
            [2, 2, 2, 2, 4, 8, 8, 8, 8, 8, 8, 8])


def ladder_valid(P, R, affine: bool) -> bool:
    """The shapes the kernels are compiled for, capacities non-decreasing."""
    if len(P) != NCLASS or len(R) != NCLASS:
        return False
    prev = 0
    for p, r in zip(P, R):
        if p not in P_ALLOWED or r not in ((2, 3, 4) if affine else (2, 4, 8)):
            return False
        cap = 2 * (p - 1) * r + 1
        if cap < prev:
            return False
        prev = cap
    return True


def candidate_ladders(affine: bool) -> list:
    """A small search space around the default: rows per lane of the narrow
    classes, where the multi-warp pipelines start, and whether R = 3 shapes
    fill the gaps between the power-of-two capacities. Every candidate ends
    on the widest shape, so that no band a default ladder takes is refused."""
    out = [default_ladder(affine)]
    if affine:
        out += [
            ([4, 8, 8, 16, 16, 32, 32, 32, 64, 64, 128, 512],
             [2, 2, 3, 2, 3, 2, 3, 4, 3, 4, 4, 4]),
            ([8, 8, 16, 16, 32, 32, 32, 64, 64, 128, 128, 512],
             [2, 3, 2, 3, 2, 3, 4, 3, 4, 3, 4, 4]),
            ([8, 16, 32, 32, 64, 128, 256, 512, 512, 512, 512, 512], [2, 2, 2] + [4] * 9),
            ([4, 8, 16, 32, 32, 64, 128, 256, 512, 512, 512, 512], [2, 2, 2, 2] + [4] * 8),
        ]
    else:
        out += [
            ([4, 8, 16, 32, 32, 64, 128, 256, 512, 512, 512, 512], [4, 4, 4, 4] + [8] * 8),
            ([4, 8, 16, 32, 64, 128, 256, 512, 512, 512, 512, 512], [8] * 12),
        ]
    assert all(ladder_valid(P, R, affine) for P, R in out)
    return out


def set_ladder(ctx: Context, affine: bool, P, R):
    p = np.ascontiguousarray(P, np.int32)
    r = np.ascontiguousarray(R, np.int32)
    check(_lib.load().poyalgn_set_ladder(ctx.handle, int(affine), _ptr(p), _ptr(r)))


def get_ladder(ctx: Context, affine: bool):
    p = np.zeros(NCLASS, np.int32)
    r = np.zeros(NCLASS, np.int32)
    check(_lib.load().poyalgn_get_ladder(ctx.handle, int(affine), _ptr(p), _ptr(r)))
    return p.tolist(), r.tolist()


def autotune(ctx: Context, cm: CostMatrix, pairs, candidates=None, reps: int = 2) -> dict:
    """Time candidate ladders on `pairs` and keep the fastest on `ctx`."""
    pk = pairs if isinstance(pairs, PackedPairs) else pack_pairs(pairs)
    cands = candidates or candidate_ladders(cm.affine)
    cp = np.ascontiguousarray([c[0] for c in cands], np.int32)
    cr = np.ascontiguousarray([c[1] for c in cands], np.int32)
    ms = np.zeros(len(cands), np.float32)
    best = np.zeros(1, np.int32)
    check(_lib.load().poyalgn_autotune(ctx.handle, cm.handle, pk.npairs, _ptr(pk.seqs),
                                       _ptr(pk.offa), _ptr(pk.lena), _ptr(pk.offb),
                                       _ptr(pk.lenb), len(cands), _ptr(cp), _ptr(cr), reps,
                                       _ptr(ms), _ptr(best)))
    b = int(best[0])
    return {"best": b, "ladder": cands[b], "ms": ms.tolist()}
