"""Band-doubling schedule arithmetic for throughput accounting.

The band of every doubling iteration is a deterministic function of the
pair's lengths, the cost matrix's smallest positive cost and (linear) the
plane choice, so the cells a pair's fill computed follow from the number of
iterations the GPU reports (`passes`). Rules as in algn_newkk_test
(src/algn.c:1063-1114), algn_newkk_test_aff (src/algn.c:2185-2306) and
algn_fill_plane_2 (src/algn.c:1134-1177).
"""
from __future__ import annotations

import numpy as np


def _sum_min_shift(m1: np.ndarray, c: np.ndarray, cap: np.ndarray) -> np.ndarray:
    """sum_{i=1}^{m1} min(cap, i + c) for vectors (all int64)."""
    # i + c <= cap  <=>  i <= cap - c
    lim = np.clip(cap - c, 0, m1)
    s1 = lim * (lim + 1) // 2 + c * lim
    s2 = (m1 - lim) * cap
    return s1 + s2


def _sum_max_shift(m1: np.ndarray, k: np.ndarray) -> np.ndarray:
    """sum_{i=1}^{m1} max(0, i - k)."""
    t = np.clip(m1 - k, 0, None)
    return t * (t + 1) // 2


def band_cells(m, n, newk, affine: bool) -> np.ndarray:
    """Cells filled by one band iteration (rows 1..m-1) for vectors m <= n."""
    m = np.asarray(m, np.int64)
    n = np.asarray(n, np.int64)
    k = np.asarray(newk, np.int64)
    D = n - m
    m1 = m - 1
    # e_i = min(n-1, i + D + k) for both models (the affine right edge is the
    # same column set), s_i = max(0, i - k)
    e_sum = _sum_min_shift(m1, D + k, n - 1)
    s_sum = _sum_max_shift(m1, k)
    return e_sum - s_sum + m1


def unstoppable_passes(la, lb, mnz: int, affine: bool) -> np.ndarray:
    """Leading doubling iterations that cannot end the doubling: a pass's gap
    count is at least n - m, so its test needs T >= 3 (n - m) + 4 (linear)
    or + 2 (affine) unless the band covers the plane. The library counts
    these as run without filling them (linear pairs off the full plane and
    gap-free affine pairs on the lean cell)."""
    la = np.asarray(la, np.int64)
    lb = np.asarray(lb, np.int64)
    m = np.minimum(la, lb)
    n = np.maximum(la, lb)
    d = n - m
    T = (d + 1) * mnz
    thr = 3 * d + (2 if affine else 4)
    s = np.zeros(len(m), np.int64)
    for it in range(39):
        cov = ((2 * T - d) // 2 - (n - 1 if affine else n) + 1) >= 0
        step = (s == it) & (T > 0) & (T < thr) & ~cov
        if not step.any():
            break
        s[step] += 1
        T = np.where(step, 2 * T, T)
    return s


def cells_computed(la, lb, passes, mnz: int, affine: bool, full=None,
                   skipped=None) -> np.ndarray:
    """Cells filled over all doubling iterations of each pair (`skipped`:
    per pair, leading iterations counted in `passes` but not filled)."""
    la = np.asarray(la, np.int64)
    lb = np.asarray(lb, np.int64)
    passes = np.asarray(passes, np.int64)
    m = np.minimum(la, lb)
    n = np.maximum(la, lb)
    total = np.zeros(len(m), np.int64)
    if full is not None:
        full = np.asarray(full, bool)
        total[full] = (m[full] - 1) * n[full]
    else:
        full = np.zeros(len(m), bool)
    skipped = np.zeros(len(m), np.int64) if skipped is None else np.asarray(skipped, np.int64)
    T = (n - m + 1) * mnz
    for it in range(int(passes.max()) if len(passes) else 0):
        if not ((passes > it) & ~full).any():
            break
        live = (passes > it) & ~full & (it >= skipped)
        p = (T - (n - m)) // 2
        kmax = (m - 2) if affine else (m - 1)
        newk = np.minimum(p, kmax)
        c = band_cells(m, n, newk, affine)
        total[live] += c[live]
        T = T * 2
    return total


def linear_full_plane(la, lb, gaps_a, gaps_b) -> np.ndarray:
    """algn_fill_plane_2's plane choice with the facade's deltawh."""
    la = np.asarray(la, np.int64)
    lb = np.asarray(lb, np.int64)
    m = np.minimum(la, lb)
    n = np.maximum(la, lb)
    gaps = np.maximum(np.asarray(gaps_a), np.asarray(gaps_b))
    lower = m // 10
    dw = np.where((m - n) < lower, lower // 2, 2)
    height = np.minimum((m - n) + 50 + gaps + dw, m)
    full = np.where(2 * m >= 3 * n, True,
                    np.where(2 * height < m, False, 8 >= m - height))
    return full.astype(bool)
