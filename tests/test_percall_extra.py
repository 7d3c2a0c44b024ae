"""The remaining per-call externals of the drop-in boundary:
algn_CAML_limit_2, algn_CAML_backtrace_2d_limit, algn_CAML_verify_2 and
seq_CAML_median_2_no_gaps.

* CPU: the identity the library's poyalgn_limit_2 relies on (limit_2 is
  simple_2 with deltawh = w + (s1_len - s2_len) - (l1 - l2)) checked on the
  compiled reference itself, and the library's verify / no-gap-median code
  (pa_core.cuh, through the host replay) against the reference;
* GPU: the C-ABI entry points against the same expectations.
"""
import ctypes as C

import numpy as np
import pytest

from cases import AFF_TCM, STD_TCM, edge_pairs, random_pairs
from oracle_lib import Oracle, available

_P = C.c_void_p


def _p(a):
    return a.ctypes.data_as(_P)


def _aligned_pairs(oracle, cm, affine, rng, n=60):
    """Aligned pairs as DOS.median produces them, plus random state pairs."""
    out = []
    for a, b in edge_pairs()[:16] + random_pairs(rng, n, maxlen=200):
        try:
            r = oracle.median(cm, a, b, affine)
        except Exception:
            continue
        out.append((r.ea, r.eb))
    for _ in range(20):
        L = int(rng.integers(1, 60))
        x = rng.choice([1, 2, 4, 8, 16, 17, 3, 15], L).astype(np.uint8)
        y = rng.choice([1, 2, 4, 8, 16, 24, 5], L).astype(np.uint8)
        out.append((x, y))
    return out


@pytest.mark.skipif(not available("ref"), reason="reference build absent")
def test_reference_limit_2_is_simple_2_with_mapped_deltawh():
    ref = Oracle("ref")
    lib = ref.lib
    cm = ref.cm(tcm=STD_TCM)
    rng = np.random.default_rng(5)
    n = 0
    # the shorter sequence first, as algn_fill_plane_2 requires (:1139)
    for a, b in random_pairs(rng, 160, maxlen=300):
        for s1, s2 in [(a, b) if len(a) <= len(b) else (b, a)]:
            l1, l2 = len(s1), len(s2)
            w = int(rng.integers(0, 30))
            s1_len = int(rng.integers(1, l1 + 1))
            s2_len = int(rng.integers(1, l2 + 1))
            c1, c2 = C.c_int(), C.c_int()
            assert lib.ref_limit_2(cm, ref._ws, _p(s1), l1, _p(s2), l2, w, 7, 0, 0,
                                   s1_len, s2_len, C.byref(c1)) == 0
            dwh = w + (s1_len - s2_len) - (l1 - l2)
            assert lib.ref_simple_2(cm, ref._ws, _p(s1), l1, _p(s2), l2, dwh,
                                    C.byref(c2)) == 0
            assert c1.value == c2.value, (l1, l2, w, s1_len, s2_len)
            n += 1
    assert n >= 100


@pytest.fixture(scope="module")
def emul():
    from conftest import build_emulator
    lib = C.CDLL(build_emulator())
    lib.pa_emul_new.restype = _P
    lib.pa_emul_new.argtypes = [_P, C.c_int, C.c_int]
    lib.pa_emul_free.argtypes = [_P]
    return lib


@pytest.mark.skipif(not available("ref"), reason="reference build absent")
@pytest.mark.parametrize("tcm,go", [(STD_TCM, 0), (AFF_TCM, 3)])
def test_verify_and_nogap_median_match_reference(oracle, emul, tcm, go):
    ref = Oracle("ref")
    rcm = ref.cm(tcm=tcm, gap_open=go)
    flat = np.ascontiguousarray(np.asarray(tcm, np.int32).reshape(-1))
    h = _P(emul.pa_emul_new(_p(flat), 5, go))
    rng = np.random.default_rng(9 + go)
    for x, y in _aligned_pairs(oracle, oracle.cm(tcm=tcm, gap_open=go), go > 0, rng):
        x = np.ascontiguousarray(x, np.uint8)
        y = np.ascontiguousarray(y, np.uint8)
        L = len(x)
        out_r, out_e = np.zeros(L + 1, np.uint8), np.zeros(L + 1, np.uint8)
        cost, n = C.c_int(), C.c_int()
        assert ref.lib.ref_verify_and_nogap(rcm, _p(x), _p(y), L, C.byref(cost), _p(out_r),
                                            C.byref(n)) == 0
        res = np.zeros(3, np.int32)
        emul.pa_emul_aligned_extra(h, _p(x), _p(y), L, _p(res), _p(out_e))
        assert res[0] == cost.value
        assert res[1] == n.value and np.array_equal(out_e[:n.value], out_r[:n.value])
    emul.pa_emul_free(h)


@pytest.mark.gpu
@pytest.mark.parametrize("tcm,go", [(STD_TCM, 0), (AFF_TCM, 3)])
def test_gpu_verify_and_nogap_median(ctx, oracle, emul, tcm, go):
    import poy5_gb300 as pg
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    flat = np.ascontiguousarray(np.asarray(tcm, np.int32).reshape(-1))
    h = _P(emul.pa_emul_new(_p(flat), 5, go))
    al = pg.Align(ctx)
    rng = np.random.default_rng(19 + go)
    for x, y in _aligned_pairs(oracle, oracle.cm(tcm=tcm, gap_open=go), go > 0, rng, 30):
        x = np.ascontiguousarray(x, np.uint8)
        y = np.ascontiguousarray(y, np.uint8)
        res = np.zeros(3, np.int32)
        out = np.zeros(len(x) + 1, np.uint8)
        emul.pa_emul_aligned_extra(h, _p(x), _p(y), len(x), _p(res), _p(out))
        assert al.verify_2(x, y, cm) == res[0]
        assert np.array_equal(al.median_2_no_gaps(x, y, cm), out[:res[1]])
    emul.pa_emul_free(h)


@pytest.mark.gpu
def test_gpu_limit_2_and_backtrace_limit(ctx, oracle):
    import poy5_gb300 as pg
    cm = pg.CostMatrix.of_list(ctx, STD_TCM, 0)
    ocm = oracle.cm(tcm=STD_TCM)
    al = pg.Align(ctx)
    rng = np.random.default_rng(23)
    for a, b in random_pairs(rng, 30, maxlen=300):
        s1, s2 = (a, b) if len(a) <= len(b) else (b, a)
        l1, l2 = len(s1), len(s2)
        w, s1_len, s2_len = int(rng.integers(0, 30)), int(rng.integers(1, l1 + 1)), l2
        got = al.limit_2(s1, s2, cm, w, 0, 0, 0, s1_len, s2_len)
        want = oracle.simple_2(ocm, s1, s2, w + (s1_len - s2_len) - (l1 - l2))
        assert got == want
        r1, r2 = al.backtrace_2d_limit(s1, s2, cm, 0, 0, l1, l2, 0)
        o1, o2 = oracle.backtrace_2d(ocm, s1, s2, 0)
        assert np.array_equal(r1, o1) and np.array_equal(r2, o2)


@pytest.mark.gpu
def test_gpu_backtrace_limit_interior_starts(ctx, emul):
    """backtrace_2d_limit from interior starts on the GPU against the host
    replay of the same walk (pinned to the compiled reference on the CPU by
    test_limit_walk_matches_reference): equal pairs where the walk stays on
    written cells, POYALGN_EUNSUPPORTED / POYALGN_EINVAL where it does not."""
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    cm = pg.CostMatrix.of_list(ctx, STD_TCM, 0)
    flat = np.ascontiguousarray(np.asarray(STD_TCM, np.int32).reshape(-1))
    h = _P(emul.pa_emul_new(_p(flat), 5, 0))
    al = pg.Align(ctx)
    rng = np.random.default_rng(37)
    seen = {0: 0, -14: 0, -15: 0}
    for a, b in edge_pairs()[:12] + random_pairs(rng, 40, maxlen=400):
        s1, s2 = (a, b) if len(a) <= len(b) else (b, a)
        s1 = np.ascontiguousarray(s1, np.uint8)
        s2 = np.ascontiguousarray(s2, np.uint8)
        l1, l2 = len(s1), len(s2)
        w, s1_len = int(rng.integers(0, 30)), int(rng.integers(1, l1 + 1))
        al.limit_2(s1, s2, cm, w, 0, 0, 0, s1_len, l2)
        dwh = w + (s1_len - l2) - (l1 - l2)
        for st1, st2, a1, a2 in _limit_starts(rng, l1, l2, 5):
            swaped = int(rng.integers(0, 2))
            cap = l1 + l2 + 4
            e1, e2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
            n, cost = C.c_int(), C.c_int()
            st = emul.pa_emul_limit_walk(h, _p(s1), l1, _p(s2), l2, dwh, st1, st2, a1, a2,
                                         swaped, _p(e1), _p(e2), cap, C.byref(n),
                                         C.byref(cost))
            seen[st] += 1
            if st == 0:
                r1, r2 = al.backtrace_2d_limit(s1, s2, cm, st1, st2, a1, a2, swaped)
                L = n.value
                assert np.array_equal(r1, e1[cap - L:]) and np.array_equal(r2, e2[cap - L:])
            else:
                with pytest.raises(pg.PoyAlgnError) as ei:
                    al.backtrace_2d_limit(s1, s2, cm, st1, st2, a1, a2, swaped)
                assert ei.value.code == (_lib.EUNSUPPORTED if st == -14 else _lib.EINVAL)
    emul.pa_emul_free(h)
    assert seen[0] >= 100 and seen[-14] >= 5, seen


def _limit_starts(rng, l1, l2, n):
    """Start cells for backtrace_2d_limit: the last cell, interior cells of
    both sequences from the origin, and windows that start past it."""
    out = [(0, 0, l1, l2)]
    for _ in range(n):
        a1 = int(rng.integers(1, l1 + 1))
        a2 = int(rng.integers(1, l2 + 1))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            out.append((0, 0, a1, a2))
        elif kind == 1 and a2 > 1:
            st2 = int(rng.integers(0, a2))
            out.append((0, st2, a1, a2 - st2))
        elif a1 > 1:
            st1 = int(rng.integers(0, a1))
            out.append((st1, 0, a1 - st1, a2))
    return out


@pytest.mark.skipif(not available("ref"), reason="reference build absent")
def test_limit_walk_matches_reference(emul):
    """backtrace_2d_limit from interior starts (lin_limit_walk through the
    host replay) against the compiled reference after the same simple_2
    fill. Starts whose walk stays on cells the last fill wrote must match
    byte for byte; the others must be refused (status -14 / -15), never
    guessed: the reference reads leftovers of earlier alignments there."""
    ref = Oracle("ref")
    rcm = ref.cm(tcm=STD_TCM)
    flat = np.ascontiguousarray(np.asarray(STD_TCM, np.int32).reshape(-1))
    h = _P(emul.pa_emul_new(_p(flat), 5, 0))
    rng = np.random.default_rng(31)
    matched = refused = 0
    for a, b in edge_pairs() + random_pairs(rng, 80, maxlen=300):
        s1, s2 = (a, b) if len(a) <= len(b) else (b, a)
        s1 = np.ascontiguousarray(s1, np.uint8)
        s2 = np.ascontiguousarray(s2, np.uint8)
        l1, l2 = len(s1), len(s2)
        dwh = int(rng.integers(0, 40))
        for st1, st2, a1, a2 in _limit_starts(rng, l1, l2, 6):
            swaped = int(rng.integers(0, 2))
            cap = l1 + l2 + 4
            e1, e2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
            n, cost = C.c_int(), C.c_int()
            st = emul.pa_emul_limit_walk(h, _p(s1), l1, _p(s2), l2, dwh, st1, st2, a1, a2,
                                         swaped, _p(e1), _p(e2), cap, C.byref(n),
                                         C.byref(cost))
            if st != 0:
                assert st in (-14, -15), st
                refused += 1
                continue
            c, rn = C.c_int(), C.c_int()
            assert ref.lib.ref_simple_2(rcm, ref._ws, _p(s1), l1, _p(s2), l2, dwh,
                                        C.byref(c)) == 0
            assert c.value == cost.value
            r1, r2 = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
            assert ref.lib.ref_backtrace_2d_limit(rcm, ref._ws, _p(s1), l1, _p(s2), l2, st1,
                                                  st2, a1, a2, swaped, _p(r1), _p(r2), cap,
                                                  C.byref(rn)) == 0
            L = n.value
            assert rn.value == L, (l1, l2, st1, st2, a1, a2)
            assert np.array_equal(e1[cap - L:], r1[:L]) and np.array_equal(e2[cap - L:], r2[:L])
            matched += 1
    emul.pa_emul_free(h)
    assert matched >= 300 and refused >= 10, (matched, refused)
