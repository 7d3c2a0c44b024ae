"""Three-sequence alignment: Sequence.Align.align_3_powell -> powell_3D_align
(src/sequence.ml:1309-1321, src/ukkCommon.c:109-150, src/ukk.checkp.c).

CPU: the oracle restatement (oracle/poy_ukk3.c) against the golden fixture
made from the reference build, and against the reference build itself where
it is present; the device machine (pa_ukk3.cuh, compiled for the host into
the test emulator) against the oracle, with windows small enough to force the
reruns the driver makes.
GPU: poyalgn_powell_3d and poyalgn_powell_3d_batch against the fixture and
the oracle, window reruns, budget splits and the per-triple errors.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from oracle_lib import Oracle, available

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "golden_powell3d.npz")
G = 16


def golden():
    z = np.load(FIXTURE)
    out = []
    for k in range(len(z["cost"])):
        seqs = tuple(z[n][z[n + "_off"][k]:z[n + "_off"][k + 1]] for n in ("a", "b", "c"))
        al = tuple(z[n][z[n + "_off"][k]:z[n + "_off"][k + 1]] for n in ("ra", "rb", "rc"))
        out.append((seqs, tuple(int(x) for x in z["costs"][k]), int(z["cost"][k]), al))
    return out


def random_triples(rng, n, maxlen=60):
    def mut(s, div):
        out = []
        for x in s:
            r = rng.random()
            if r < div / 4:
                continue
            if r < div / 2:
                out.append(int(rng.choice([1, 2, 4, 8])))
            out.append(x if rng.random() > div else int(rng.choice([1, 2, 4, 8])))
        return out

    cases = []
    for _ in range(n):
        L = int(rng.integers(0, maxlen))
        div = float(rng.choice([0.02, 0.1, 0.3, 0.6]))
        base = rng.choice([1, 2, 4, 8], L).tolist()
        t = []
        for _ in range(3):
            s = [G] + mut(base, div)
            for i in range(1, len(s)):
                if rng.random() < 0.05:
                    s[i] |= int(rng.choice([1, 2, 4, 8, 16]))
            t.append(np.array(s, np.uint8))
        c = (int(rng.choice([1, 2, 3])), int(rng.choice([0, 0, 1, 2, 3])),
             int(rng.choice([1, 2, 3])))
        cases.append((tuple(t), c))
    return cases


def same(r, cost, al):
    return r[0] == cost and all(np.array_equal(x, y) for x, y in zip(r[1:], al))


# ---- CPU: the oracle -------------------------------------------------------

def test_oracle_matches_golden_fixture(oracle):
    cases = golden()
    assert len(cases) >= 90
    for k, (seqs, c, cost, al) in enumerate(cases):
        assert same(oracle.powell_3d(*seqs, *c), cost, al), k


@pytest.mark.skipif(not available("ref"), reason="reference build absent")
def test_oracle_matches_reference_build(oracle):
    ref = Oracle("ref")
    rng = np.random.default_rng(5150)
    for k, (seqs, c) in enumerate(random_triples(rng, 60, maxlen=45)):
        r = ref.powell_3d(*seqs, *c)
        assert same(oracle.powell_3d(*seqs, *c), r[0], r[1:]), k


def test_oracle_rejects_a_position_without_a_base(oracle):
    from oracle_lib import OracleError
    with pytest.raises(OracleError):
        oracle.powell_3d([G, 16, 1], [G, 1], [G, 1], 1, 0, 2)


def test_oracle_batch_matches_single_calls(oracle):
    from poy5_gb300.three_d import pack_triples
    rng = np.random.default_rng(99)
    cases = random_triples(rng, 24, maxlen=40)
    c = (1, 0, 2)
    seqs, off, lens, out_off, cap = pack_triples([t for t, _ in cases])
    res = oracle.powell_3d_batch(seqs, off, lens, out_off, *c, nthreads=4)
    for k, (t, _) in enumerate(cases):
        r = oracle.powell_3d(*t, *c)
        e = int(out_off[k] + cap[k])
        n = int(res["rlen"][k])
        got = tuple(res[x][e - n:e] for x in ("ra", "rb", "rc"))
        assert res["status"][k] == 0 and same(r, int(res["cost"][k]), got), k


# ---- CPU: the device machine, emulated ---------------------------------------

def _emul():
    from conftest import build_emulator
    lib = C.CDLL(build_emulator())
    lib.pa_emul_powell_3d.restype = C.c_int
    return lib


def emul_run(lib, seqs, c, D):
    a, b, cc = (np.ascontiguousarray(x, np.uint8) for x in seqs)
    cap = len(a) + len(b) + len(cc)
    ra, rb, rc = (np.zeros(cap, np.uint8) for _ in range(3))
    n, cost, steps = C.c_int(), C.c_int(), C.c_longlong()
    P = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
    st = lib.pa_emul_powell_3d(P(a), len(a), P(b), len(b), P(cc), len(cc), *c, D, P(ra), P(rb),
                               P(rc), cap, C.byref(n), C.byref(cost), C.byref(steps))
    k = n.value
    return st, cost.value, (ra[cap - k:], rb[cap - k:], rc[cap - k:])


def emul_with_reruns(lib, seqs, c, D):
    """The driver's policy: double the window after a window, stack or step
    status until it covers every diagonal."""
    full = max(len(s) - 1 for s in seqs)
    reruns = 0
    while True:
        st, cost, al = emul_run(lib, seqs, c, D)
        if st in (1, 2, 3) and D < full:
            D = min(2 * D, full)
            reruns += 1
            continue
        return st, cost, al, reruns


def test_emulated_machine_matches_golden_fixture():
    lib = _emul()
    for k, (seqs, c, cost, al) in enumerate(golden()):
        st, got, gal, _ = emul_with_reruns(lib, seqs, c, 16)
        assert st == 0 and got == cost, k
        assert all(np.array_equal(x, y) for x, y in zip(gal, al)), k


def test_emulated_machine_reruns_from_tiny_windows(oracle):
    lib = _emul()
    rng = np.random.default_rng(2718)
    total = 0
    for k, (seqs, c) in enumerate(random_triples(rng, 40, maxlen=50)):
        r = oracle.powell_3d(*seqs, *c)
        st, got, gal, reruns = emul_with_reruns(lib, seqs, c, 1)
        total += reruns
        assert st == 0 and same(r, got, gal), k
    assert total > 20


# ---- GPU ------------------------------------------------------------------

@pytest.fixture(scope="module")
def ctx():
    import poy5_gb300 as pg
    return pg.Context(0)


@pytest.mark.gpu
def test_gpu_batch_matches_golden_fixture(ctx):
    import poy5_gb300 as pg
    cases = golden()
    by_cost = {}
    for seqs, c, cost, al in cases:
        by_cost.setdefault(c, []).append((seqs, cost, al))
    for c, items in by_cost.items():
        res = pg.powell_3d_batch(ctx, [s for s, _, _ in items], *c)
        for k, (_, cost, al) in enumerate(items):
            assert res.status[k] == 0 and res.cost[k] == cost, (c, k)
            assert all(np.array_equal(x, y) for x, y in zip(res.aligned(k), al)), (c, k)


@pytest.mark.gpu
def test_gpu_single_call_matches_golden_and_ends_at_capacity(ctx):
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    lib = _lib.load()
    for seqs, c, cost, al in golden()[::7]:
        got = pg.align_3_powell(ctx, *seqs, *c)
        assert got[3] == cost
        assert all(np.array_equal(x, y) for x, y in zip(got[:3], al))
        # the seq_prepend layout: a larger buffer is filled at its end
        a, b, cc = (np.ascontiguousarray(x, np.uint8) for x in seqs)
        cap = len(a) + len(b) + len(cc) + 5
        ra, rb, rc = (np.full(cap, 99, np.uint8) for _ in range(3))
        n, d = C.c_int32(), C.c_int32()
        P = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
        _lib.check(lib.poyalgn_powell_3d(ctx.handle, P(a), len(a), P(b), len(b), P(cc), len(cc),
                                         *c, P(ra), P(rb), P(rc), cap, C.byref(n), C.byref(d)))
        k = n.value
        assert np.array_equal(ra[cap - k:], al[0]) and (ra[:cap - k] == 99).all()


@pytest.mark.gpu
def test_gpu_batch_matches_oracle_with_window_reruns(ctx, oracle):
    import poy5_gb300 as pg
    rng = np.random.default_rng(8086)
    # divergent triples: their costs outgrow the first window
    cases = random_triples(rng, 96, maxlen=70)
    c = (1, 2, 1)
    triples = [t for t, _ in cases]
    res = pg.powell_3d_batch(ctx, triples, *c)
    assert res.rounds >= 2
    for k, t in enumerate(triples):
        r = oracle.powell_3d(*t, *c)
        assert res.status[k] == 0 and same(r, int(res.cost[k]), res.aligned(k)), k


@pytest.mark.gpu
def test_gpu_budget_splits_into_rounds(ctx, oracle):
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    w = wl.readjust_triples(n_triples=48, lo=60, hi=120)
    one = pg.powell_3d_batch(ctx, w.triples, w.mm, w.go, w.ge)
    small = pg.powell_3d_batch(ctx, w.triples, w.mm, w.go, w.ge, budget_bytes=8 << 20)
    pg.powell_3d_batch(ctx, [], w.mm, w.go, w.ge, budget_bytes=0)
    assert small.rounds > one.rounds
    assert np.array_equal(one.cost, small.cost)
    for k, t in enumerate(w.triples[:16]):
        r = oracle.powell_3d(*t, w.mm, w.go, w.ge)
        assert same(r, int(small.cost[k]), small.aligned(k)), k
        assert all(np.array_equal(x, y) for x, y in zip(one.aligned(k), small.aligned(k)))


@pytest.mark.gpu
def test_gpu_readjust_workload_matches_oracle(ctx, oracle):
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    from poy5_gb300.three_d import pack_triples
    w = wl.readjust_triples(n_triples=256)
    res = pg.powell_3d_batch(ctx, w.triples, w.mm, w.go, w.ge)
    seqs, off, lens, out_off, cap = pack_triples(w.triples)
    ref = oracle.powell_3d_batch(seqs, off, lens, out_off, w.mm, w.go, w.ge)
    assert (ref["status"] == 0).all() and (res.status == 0).all()
    assert np.array_equal(ref["cost"], res.cost)
    assert np.array_equal(ref["rlen"], res.rlen)
    for name, got in (("ra", res.ra), ("rb", res.rb), ("rc", res.rc)):
        for k in range(len(w.triples)):
            e, n = int(out_off[k] + cap[k]), int(res.rlen[k])
            assert np.array_equal(ref[name][e - n:e], got[e - n:e]), (name, k)


@pytest.mark.gpu
def test_gpu_per_triple_errors(ctx):
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    good = ([G, 1, 2], [G, 1, 2], [G, 1, 4])
    bad_base = ([G, 16, 1], [G, 1], [G, 1])   # POY: "This is impossible!"
    empty = ([], [G, 1], [G, 1])
    res = pg.powell_3d_batch(ctx, [good, bad_base, empty, good], 1, 0, 2, raise_on_error=False)
    assert list(res.status) == [0, -7, -4, 0]
    assert res.cost[0] == res.cost[3] and res.cost[1] == -1
    with pytest.raises(_lib.PoyAlgnError):
        pg.powell_3d_batch(ctx, [good], 0, 0, 2)     # mismatch cost 0
    with pytest.raises(_lib.PoyAlgnError):
        pg.powell_3d_batch(ctx, [good], 1, 20000, 2)  # past the state tables' range
    # a cost bound past 2^26 (large gap costs on long sequences) is refused per
    # triple before any launch
    G_ = [G] + [1] * 30000
    big = pg.powell_3d_batch(ctx, [(G_, G_, G_), good], 1, 9000, 9000, raise_on_error=False)
    assert list(big.status) == [-6, 0]
    with pytest.raises(_lib.PoyAlgnError):
        pg.powell_3d_batch(ctx, [bad_base], 1, 0, 2)


@pytest.mark.gpu
def test_gpu_readjust_workload_affine_costs_match_oracle(ctx, oracle):
    """The readjust triples under affine costs (mismatch 1, opening 3,
    extension 1): 16 cost planes and wider windows than the linear model."""
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    from poy5_gb300.three_d import pack_triples
    w = wl.readjust_triples(n_triples=128, lo=80, hi=200)
    mm, go, ge = 1, 3, 1
    res = pg.powell_3d_batch(ctx, w.triples, mm, go, ge)
    seqs, off, lens, out_off, cap = pack_triples(w.triples)
    ref = oracle.powell_3d_batch(seqs, off, lens, out_off, mm, go, ge)
    assert (ref["status"] == 0).all() and (res.status == 0).all()
    assert np.array_equal(ref["cost"], res.cost)
    assert np.array_equal(ref["rlen"], res.rlen)
    for k in range(len(w.triples)):
        e, n = int(out_off[k] + cap[k]), int(res.rlen[k])
        for name, got in (("ra", res.ra), ("rb", res.rb), ("rc", res.rc)):
            assert np.array_equal(ref[name][e - n:e], got[e - n:e]), (name, k)
