"""Algn_Newkk (src/newkkonen.c), affine: POY's own banded aligner behind
Sequence.NewkkAlign.align_2, used by DOS.median when use_ukk is set.

* the oracle's restatement against the golden fixture generated from the
  reference build (always) and against the reference itself on random pairs
  (where oracle/_ref exists);
* the library (C ABI) against the oracle: the per-call stubs
  newkkonen_CAML_algn_affine / _backtrace_affine and the batched DOS.median.
"""
from __future__ import annotations

import numpy as np
import pytest

import golden_lib
from cases import AFF_TCM, edge_pairs, random_pairs
from oracle_lib import Oracle, OracleError, available


def _same(r, p):
    return (r.cost == p.cost and r.maxcost == p.maxcost
            and np.array_equal(r.ea, p.ea) and np.array_equal(r.eb, p.eb)
            and np.array_equal(r.median, p.median)
            and np.array_equal(r.medianwg, p.medianwg))


@pytest.mark.parametrize("name", golden_lib.NEWKK_NAMES)
def test_oracle_newkk_matches_golden(oracle, name):
    g = golden_lib.load(name)
    cm = oracle.cm(tcm=g.tcm, gap_open=g.gap_open)
    bad = []
    for k, (a, b) in enumerate(g.pairs):
        r = oracle.newkk_median(cm, a, b)
        m = golden_lib.mismatches(g, k, r.cost, r.ea, r.eb, r.median, r.medianwg, r.maxcost)
        if m:
            bad.append((k, m))
    assert not bad, bad[:5]


@pytest.mark.skipif(not available("ref"), reason="reference build absent")
@pytest.mark.parametrize("model", [(1, 1, 3), (1, 2, 2), (2, 1, 1), (3, 2, 5)])
def test_oracle_newkk_matches_reference(oracle, model):
    ref = Oracle("ref")
    subs, indel, go = model
    tcm = [[0 if r == c else (indel if 4 in (r, c) else subs) for c in range(5)]
           for r in range(5)]
    cr, cp = ref.cm(tcm=tcm, gap_open=go), oracle.cm(tcm=tcm, gap_open=go)
    rng = np.random.default_rng(sum(model))
    pairs = edge_pairs() + random_pairs(rng, 80, maxlen=300)
    # a few long pairs: several 32-row rounds and band passes
    for L in (900, 1500):
        a = np.array([16] + list(rng.choice([1, 2, 4, 8], L)), np.uint8)
        b = a.copy()
        b[1:][rng.random(L) < 0.12] = 2
        pairs += [(a, np.concatenate([b[:L // 2], b[L // 2 + 9:]])), (b[:L - 40], a)]
    for k, (a, b) in enumerate(pairs):
        try:
            r = ref.newkk_median(cr, a, b)
        except OracleError:
            with pytest.raises(OracleError):
                oracle.newkk_median(cp, a, b)
            continue
        assert _same(r, oracle.newkk_median(cp, a, b)), (model, k)


def test_oracle_newkk_trivial_path(oracle):
    """s1_len * 100 < s2_len: trivial_algn / trivial_backtrace (indel sums,
    the shorter sequence's states first and reversed)."""
    cm = oracle.cm(tcm=AFF_TCM, gap_open=3)
    a = np.array([16, 1, 2], np.uint8)
    b = np.array([16] + [1, 2, 4, 8] * 80, np.uint8)
    cost, r1, r2, iters, _ = oracle.newkk_align(cm, a, b, 0)
    t = oracle.tables(cm)
    ind = lambda s: sum(int(t["cost"][((int(x) & 15) << t["lcm"]) + 16]) for x in s)
    assert cost == ind(a) + ind(b) and iters == 0
    assert list(r1) == [16] * len(b) + list(a[::-1])
    assert list(r2) == list(b[::-1]) + [16] * len(a)


def test_oracle_newkk_rejects_linear(oracle):
    """The reference's linear Newkk keeps a zero-cost diagonal candidate and
    its backtrace asserts (src/newkkonen.c:796, 1554): only affine."""
    cm = oracle.cm(subs=1, indel=2)
    with pytest.raises(OracleError):
        oracle.newkk_median(cm, np.array([16, 1], np.uint8), np.array([16, 2], np.uint8))


# ---- the kernel's warp schedule replayed on the host (no GPU) -------------

def _emul_newkk(lib, h, a, b):
    import ctypes as C
    a = np.ascontiguousarray(a, np.uint8)
    b = np.ascontiguousarray(b, np.uint8)
    cap = len(a) + len(b) + 2
    bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
    res = np.zeros(4, np.int32)
    cost, ps = C.c_int(), C.c_int()
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    rc = lib.pa_emul_newkk_median(h, p(a), len(a), p(b), len(b), C.byref(cost),
                                  *(p(x) for x in bufs), p(res), C.byref(ps))
    al, ml, wl, mx = (int(x) for x in res)
    return rc, cost.value, bufs[0][cap - al:], bufs[1][cap - al:], bufs[2][cap - ml:], \
        bufs[3][cap - wl:], mx


@pytest.fixture(scope="module")
def nk_emul():
    import ctypes as C
    from conftest import build_emulator
    lib = C.CDLL(build_emulator())
    lib.pa_emul_new.restype = C.c_void_p
    lib.pa_emul_new.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.pa_emul_free.argtypes = [C.c_void_p]
    return lib


def _emul_handle(lib, tcm, go):
    import ctypes as C
    flat = np.ascontiguousarray(np.asarray(tcm, np.int32).reshape(-1))
    return C.c_void_p(lib.pa_emul_new(flat.ctypes.data_as(C.c_void_p), 5, go))


def test_replay_newkk_matches_golden(nk_emul):
    g = golden_lib.load("golden_newkk")
    h = _emul_handle(nk_emul, g.tcm, g.gap_open)
    bad = []
    for k, (a, b) in enumerate(g.pairs):
        rc, cost, ea, eb, med, mwg, mx = _emul_newkk(nk_emul, h, a, b)
        m = golden_lib.mismatches(g, k, cost, ea, eb, med, mwg, mx) if rc == 0 else ["rc%d" % rc]
        if m:
            bad.append((k, m))
    nk_emul.pa_emul_free(h)
    assert not bad, bad[:5]


@pytest.mark.parametrize("model", [(1, 1, 3), (2, 1, 1), (3, 2, 5)])
def test_replay_newkk_matches_oracle(oracle, nk_emul, model):
    subs, indel, go = model
    tcm = [[0 if r == c else (indel if 4 in (r, c) else subs) for c in range(5)]
           for r in range(5)]
    cm = oracle.cm(tcm=tcm, gap_open=go)
    h = _emul_handle(nk_emul, tcm, go)
    rng = np.random.default_rng(7 + go)
    # lengths across tile boundaries (multiples of 32 +- 1) and wide bands
    pairs = random_pairs(rng, 60, maxlen=300)
    for L in (31, 32, 33, 63, 64, 65, 97):
        a = np.array([16] + list(rng.choice([1, 2, 4, 8], L - 1)), np.uint8)
        b = np.array([16] + list(rng.choice([1, 2, 4, 8], L + int(rng.integers(0, 40)))), np.uint8)
        pairs += [(a, b), (b, a)]
    for k, (a, b) in enumerate(pairs):
        try:
            r = oracle.newkk_median(cm, a, b)
        except OracleError:
            continue
        rc, cost, ea, eb, med, mwg, mx = _emul_newkk(nk_emul, h, a, b)
        assert rc == 0, (k, rc)
        assert cost == r.cost and mx == r.maxcost, k
        assert np.array_equal(ea, r.ea) and np.array_equal(eb, r.eb), k
        assert np.array_equal(med, r.median) and np.array_equal(mwg, r.medianwg), k
    nk_emul.pa_emul_free(h)


# ---- the CUDA library (C ABI) against the reference and the oracle ---------

def _check_batch(res, want, tag):
    bad = []
    for k, r in enumerate(want):
        d = res.pair(k)
        if res.status[k] != 0:
            bad.append((k, "status", int(res.status[k])))
            continue
        if (d.cost, d.maxcost) != (r.cost, r.maxcost):
            bad.append((k, "cost", d.cost, r.cost))
        elif not (np.array_equal(d.aligned_a, r.ea) and np.array_equal(d.aligned_b, r.eb)):
            bad.append((k, "alignment"))
        elif not (np.array_equal(d.median, r.median) and np.array_equal(d.median_wg, r.medianwg)):
            bad.append((k, "median"))
    assert not bad, (tag, bad[:5])


@pytest.mark.gpu
def test_gpu_newkk_batch_matches_golden(ctx):
    import poy5_gb300 as pg
    g = golden_lib.load("golden_newkk")
    cm = pg.CostMatrix.of_list(ctx, g.tcm, g.gap_open)
    res = pg.newkk_median_batch(ctx, cm, g.pairs)
    bad = []
    for k in range(len(g.pairs)):
        d = res.pair(k)
        m = golden_lib.mismatches(g, k, d.cost, d.aligned_a, d.aligned_b, d.median,
                                  d.median_wg, d.maxcost)
        if res.status[k] != 0 or m:
            bad.append((k, int(res.status[k]), m))
    assert not bad, bad[:5]


@pytest.mark.gpu
@pytest.mark.parametrize("model", [(1, 1, 3), (2, 1, 1)])
def test_gpu_newkk_batch_matches_oracle(ctx, oracle, model):
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    subs, indel, go = model
    tcm = [[0 if r == c else (indel if 4 in (r, c) else subs) for c in range(5)]
           for r in range(5)]
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    ocm = oracle.cm(tcm=tcm, gap_open=go)
    rng = np.random.default_rng(11 + go)
    pairs = random_pairs(rng, 150, maxlen=400) + wl.affine_pairs(n_pairs=300).pairs
    want = [oracle.newkk_median(ocm, a, b) for a, b in pairs]
    _check_batch(pg.newkk_median_batch(ctx, cm, pairs), want, model)


@pytest.mark.gpu
def test_gpu_newkk_arena_reruns(ctx, oracle):
    """A direction arena far smaller than the batch's bands: the pairs that
    do not fit are finished by further launches, with the same results."""
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    c2 = pg.Context(0)
    nk = pg.NewkkAlign(c2)
    nk.set_arena_words(1 << 23)  # the largest band here is ~3 M words
    cm = pg.CostMatrix.of_list(c2, AFF_TCM, 3)
    ocm = oracle.cm(tcm=AFF_TCM, gap_open=3)
    pairs = wl.affine_pairs(n_pairs=400).pairs
    want = [oracle.newkk_median(ocm, a, b) for a, b in pairs]
    res = pg.newkk_median_batch(c2, cm, pairs)
    assert c2.last_launches() > 1
    _check_batch(res, want, "small arena")


@pytest.mark.gpu
def test_gpu_newkk_per_call_stubs(ctx, oracle):
    """newkkonen_CAML_algn_affine + _backtrace_affine through NewkkAlign.align_2
    (both argument orders), get_k, and the misuse errors."""
    import poy5_gb300 as pg
    cm = pg.CostMatrix.of_list(ctx, AFF_TCM, 3)
    ocm = oracle.cm(tcm=AFF_TCM, gap_open=3)
    nk = pg.NewkkAlign(ctx)
    rng = np.random.default_rng(3)
    for a, b in edge_pairs()[:12] + random_pairs(rng, 20, maxlen=200):
        if len(a) == 1 and len(b) == 1:
            continue
        try:
            r = oracle.newkk_median(ocm, a, b)
        except OracleError:
            continue
        pa, pb, cost = nk.align_2(a, b, cm)
        assert cost == r.cost
        assert np.array_equal(pa, r.ea) and np.array_equal(pb, r.eb)
        assert 0 <= nk.get_k() < max(len(a), len(b))
    with pytest.raises(pg.PoyAlgnError):
        nk.cost2_affine(np.array([16, 1, 2, 4], np.uint8), np.array([16, 1], np.uint8), cm, 0)
    lin = pg.CostMatrix.of_list(ctx, [[0 if r == c else 1 for c in range(5)] for r in range(5)], 0)
    with pytest.raises(pg.PoyAlgnError):
        pg.newkk_median_batch(ctx, lin, [(np.array([16, 1], np.uint8), np.array([16, 2], np.uint8))])


@pytest.mark.gpu
def test_gpu_newkk_distance(ctx, oracle):
    """DOS.distance with use_ukk: missing_distance for an all-gap sequence,
    otherwise the Newkk cost of the pair (shorter first)."""
    import poy5_gb300 as pg
    cm = pg.CostMatrix.of_list(ctx, AFF_TCM, 3)
    ocm = oracle.cm(tcm=AFF_TCM, gap_open=3)
    rng = np.random.default_rng(21)
    pairs = random_pairs(rng, 60, maxlen=300)
    pairs += [(np.array([16, 16, 16], np.uint8), pairs[0][1]),
              (pairs[1][0], np.array([16], np.uint8))]
    got = pg.newkk_distance_batch(ctx, cm, pairs, missing_distance=7)
    for k, (a, b) in enumerate(pairs):
        if np.all(a == 16) or np.all(b == 16):
            assert got[k] == 7, k
            continue
        s1, s2 = (a, b) if len(a) <= len(b) else (b, a)
        assert got[k] == oracle.newkk_align(ocm, s1, s2, 0)[0], k


@pytest.mark.parametrize("model", [(1, 1, 3), (2, 1, 1), (3, 2, 5)])
def test_replay_newkk_passes_bound_and_skip(nk_emul, model):
    """Every fill of the newkk pass loop reports a larger gap counter of at
    least lenY - lenX (the bound behind the passes drive() counts as run
    without a fill), and skipping them gives the same outputs and pass
    count as running them."""
    import ctypes as C
    subs, indel, go = model
    tcm = [[0 if r == c else (indel if 4 in (r, c) else subs) for c in range(5)]
           for r in range(5)]
    lib = nk_emul
    lib.pa_emul_set_skip.argtypes = [C.c_void_p, C.c_int]
    full, skip = _emul_handle(lib, tcm, go), _emul_handle(lib, tcm, go)
    lib.pa_emul_set_skip(full, 0)
    lib.pa_emul_set_skip(skip, 1)
    rng = np.random.default_rng(30 + go)
    pairs = random_pairs(rng, 120, maxlen=400)
    for L in (33, 65, 130, 257):
        a = np.array([16] + list(rng.choice([1, 2, 4, 8], L - 1)), np.uint8)
        for extra in (0, 3, 40, 300):
            b = np.array([16] + list(rng.choice([1, 2, 4, 8], L - 1 + extra)), np.uint8)
            pairs += [(a, b), (b, a)]
    ks, gns = np.zeros(64, np.int32), np.zeros(64, np.int32)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    checked = 0
    for a, b in pairs:
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        n0, n1 = C.c_int(), C.c_int()
        nf = lib.pa_emul_newkk_passes(full, p(a), len(a), p(b), len(b), p(ks), p(gns), 64,
                                      C.byref(n0))
        if nf < 0:
            continue
        d = abs(len(a) - len(b))
        for j in range(nf):
            assert gns[j] >= d, (len(a), len(b), j, int(ks[j]), int(gns[j]))
            checked += 1
        lib.pa_emul_newkk_passes(skip, p(a), len(a), p(b), len(b), p(ks), p(gns), 64,
                                 C.byref(n1))
        assert n0.value == n1.value, (len(a), len(b))
        r0, r1 = _emul_newkk(lib, full, a, b), _emul_newkk(lib, skip, a, b)
        assert r0[0] == r1[0] and r0[1] == r1[1] and r0[-1] == r1[-1]
        for x, y in zip(r0[2:6], r1[2:6]):
            assert np.array_equal(x, y)
    lib.pa_emul_free(full)
    lib.pa_emul_free(skip)
    assert checked > 200
