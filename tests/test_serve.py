"""Serving loop: request traces on the CPU; on the GPU, that every request's
results are those of the plain store batch, alone and in a mix, and that
admission control refuses work beyond the waiting bound."""
import numpy as np
import pytest

import poy5_gb300 as pg
from poy5_gb300 import workloads as wl


def test_poisson_trace_shape():
    rng = np.random.default_rng(3)
    t = pg.poisson_trace(rng, 5000.0, 20000, np.arange(100), np.arange(100, 200))
    assert t.nreq == 20000 and t.arrival_s[0] == 0.0
    assert np.all(np.diff(t.arrival_s) >= 0)
    assert abs(t.nreq / t.arrival_s[-1] - 5000.0) < 150.0
    assert t.npairs.min() == 1 and t.npairs.max() == 64
    assert len(t.node_a) == t.npairs.sum() == len(t.node_b)
    assert np.all(t.node_b - t.node_a == 100)


def _pool(ctx, n=48, seed=11):
    w = wl.serving_pairs(n_pairs=n, seed=seed)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    store = pg.Store(ctx, 64 << 20)
    na = np.array([store.add(a) for a, _ in w.pairs], np.int32)
    nb = np.array([store.add(b) for _, b in w.pairs], np.int32)
    return w, cm, store, na, nb


@pytest.mark.gpu
def test_results_same_alone_and_in_mix(ctx, oracle):
    w, cm, store, na, nb = _pool(ctx)
    ref_med, ref_cost, _, ref_st = store.median_batch(cm, na, nb, keep=True)
    assert np.all(ref_st == 0)
    ocm = oracle.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    for k in range(4):  # the store batch itself against the oracle
        r = oracle.median(ocm, *w.pairs[k], True)
        assert r.cost == ref_cost[k]
        assert np.array_equal(store.read(int(ref_med[k])), r.median)
    srv = pg.Server(store, cm, nslots=2, max_batch_pairs=96, max_waiting_pairs=4096,
                    hbm_budget=2 << 30)
    pick = np.array([5, 17, 3, 40, 41, 8, 29], np.int32)
    alone = srv.wait(srv.submit(na[pick], nb[pick]))
    assert np.array_equal(alone.cost, ref_cost[pick]) and np.all(alone.status == 0)
    # the same request in the middle of a burst of others
    rng = np.random.default_rng(5)
    tickets, picks = [], []
    for q in range(24):
        p = pick if q == 12 else rng.integers(0, len(na), int(rng.integers(1, 20))).astype(np.int32)
        tickets.append(srv.submit(na[p], nb[p]))
        picks.append(p)
    for t, p in zip(tickets, picks):
        rep = srv.wait(t)
        assert np.all(rep.status == 0) and rep.latency_s > 0
        assert np.array_equal(rep.cost, ref_cost[p])
        for k, m in zip(p, rep.medians):
            assert np.array_equal(m, store.read(int(ref_med[k])))
    mixed = srv.wait(srv.submit(na[pick], nb[pick]))
    for x, y in zip(alone.medians, mixed.medians):
        assert np.array_equal(x, y)
    # an open-loop replay of a Poisson trace
    tr = pg.poisson_trace(rng, 3000.0, 150, na, nb, max_pairs=16)
    res = srv.replay(tr)
    assert np.all(res.served()) and np.all(res.status == 0)
    assert res.wall_s > 0 and np.all(res.latency_s > 0)
    want = ref_cost[np.searchsorted(na, tr.node_a)]
    assert np.array_equal(res.cost, want)
    st = srv.stats()
    assert st["refused"] == 0 and st["pairs"] >= int(tr.npairs.sum())
    srv.close()


@pytest.mark.gpu
def test_admission_refuses_beyond_waiting_bound(ctx):
    w, cm, store, na, nb = _pool(ctx, n=64, seed=12)
    srv = pg.Server(store, cm, nslots=1, max_batch_pairs=64, max_waiting_pairs=64,
                    hbm_budget=1 << 30)
    nreq = 12
    tr = pg.Trace(np.zeros(nreq), np.full(nreq, 64, np.int32), np.tile(na, nreq),
                  np.tile(nb, nreq))
    res = srv.replay(tr)
    refused = ~res.served()
    assert refused.sum() >= nreq // 2, res.latency_s
    assert np.all(res.status[np.repeat(refused, 64)] == 1)
    ok = np.repeat(~refused, 64)
    assert np.all(res.status[ok] == 0)
    assert srv.stats()["refused"] == int(refused.sum())
    with pytest.raises(pg.PoyAlgnError):
        srv.submit(np.zeros(65, np.int32), np.zeros(65, np.int32))  # larger than a batch
    srv.close()


@pytest.mark.gpu
def test_distance_server_matches_distance_batch(ctx):
    from poy5_gb300.serve import DISTANCE
    w, cm, store, na, nb = _pool(ctx, n=40, seed=13)
    want, st = pg.distance_batch(ctx, cm, w.pairs)
    assert np.all(st == 0)
    srv = pg.Server(store, cm, nslots=2, max_batch_pairs=64, max_waiting_pairs=4096,
                    hbm_budget=1 << 30, kind=DISTANCE)
    pick = np.array([3, 9, 27, 0], np.int32)
    alone = srv.wait(srv.submit(na[pick], nb[pick]))
    assert np.array_equal(alone.cost, want[pick])
    assert all(len(m) == 0 for m in alone.medians)
    rng = np.random.default_rng(8)
    tr = pg.poisson_trace(rng, 5000.0, 120, na, nb, max_pairs=12)
    res = srv.replay(tr)
    assert np.all(res.served()) and np.all(res.status == 0)
    assert np.array_equal(res.cost, want[np.searchsorted(na, tr.node_a)])
    srv.close()
