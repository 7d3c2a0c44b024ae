"""Speculative band passes: running a pair's first passes at once and keeping
the first that satisfies the doubling test must give exactly the results of
the sequential doubling (costs, medians, alignments, pass counts)."""
import numpy as np
import pytest

from cases import AFF_TCM, STD_TCM, edge_pairs, random_pairs
from poy5_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a.status, b.status)
    ok = a.status == 0
    for f in ("cost", "maxcost", "alen", "mlen", "wlen", "passes"):
        assert np.array_equal(getattr(a, f)[ok], getattr(b, f)[ok]), f
    for k in np.flatnonzero(ok):
        x, y = a.pair(k), b.pair(k)
        assert np.array_equal(x.median, y.median) and np.array_equal(x.aligned_a, y.aligned_a)
        assert np.array_equal(x.aligned_b, y.aligned_b) and np.array_equal(x.median_wg, y.median_wg)


@pytest.mark.parametrize("model", ["affine", "linear"])
def test_speculative_passes_match_sequential(model, oracle):
    import poy5_gb300 as pg
    rng = np.random.default_rng(71 + (model == "affine"))
    tcm, go = (AFF_TCM, 3) if model == "affine" else (STD_TCM, 0)
    # gap-free pairs speculate; gapped affine ones take the sequential path
    # in the same batch
    pairs = edge_pairs() + random_pairs(rng, 120, maxlen=900)
    w = wl.affine_pairs(n_pairs=24) if model == "affine" else wl.plain_pairs(n_pairs=24)
    pairs += w.pairs
    ctx = pg.Context(0)
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    ctx.set_speculation(0)
    ref = pg.median_batch(ctx, cm, pairs)
    ocm = oracle.cm(tcm=tcm, gap_open=go)
    for k in range(0, len(pairs), 7):  # the sequential results themselves
        if ref.status[k] != 0:
            continue
        r = oracle.median(ocm, *pairs[k], model == "affine")
        assert ref.cost[k] == r.cost and np.array_equal(ref.pair(k).median, r.median), k
    for passes in (1, 2, 4, 7):
        ctx.set_speculation(1, passes)
        _same(ref, pg.median_batch(ctx, cm, pairs))
    ctx.set_speculation(2, 4)  # auto: this batch is small enough
    _same(ref, pg.median_batch(ctx, cm, pairs))
    with pytest.raises(pg.PoyAlgnError):
        ctx.set_speculation(1, 0)
    ctx.close()


def test_speculative_distance_and_downpass():
    import poy5_gb300 as pg
    t = wl.yule_tree(n_taxa=32, root_len=600)
    ctx = pg.Context(0)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, t.subs, t.indel, t.gap_open)
    out = {}
    for mode in (0, 1):
        ctx.set_speculation(mode, 3)
        store = pg.Store(ctx, 16 << 20)
        leaves = [store.add(s) for s in t.leaves]
        res = pg.downpass(store, cm, leaves, t.left, t.right)
        meds = [store.read(int(x)) for x in res.internal_node]
        dist, st = pg.distance_batch(ctx, cm, list(zip(t.leaves[:-1], t.leaves[1:])))
        out[mode] = (res.total_cost, list(res.internal_cost), meds, dist, st)
    a, b = out[0], out[1]
    assert a[0] == b[0] and a[1] == b[1]
    assert all(np.array_equal(x, y) for x, y in zip(a[2], b[2]))
    assert np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4]) and np.all(a[4] == 0)
    ctx.close()


def test_second_sweep_matches_sequential(oracle):
    """Linear pairs of 4-9 kb (together at least 8,192 positions: the second
    speculative sweep runs the passes up to each pair's predicted final pass
    at once). With a first sweep of 1 or 2 passes the prediction comes from
    gap counts that have not settled yet, so mispredictions (a pass before
    the predicted one stops, or none does) take the rerun paths. Results,
    pass counts and distances must equal the sequential doubling's."""
    import poy5_gb300 as pg
    rng = np.random.default_rng(404)
    pairs = []
    for t in range(20):
        L = int(rng.integers(4200, 9000))
        core = wl.random_bases(rng, L)
        sub, ind = [(0.05, 0.01), (0.15, 0.02), (0.3, 0.06), (0.1, 0.1)][t % 4]
        pairs.append((wl.with_gap(core), wl.with_gap(wl.mutate(rng, core, sub, ind))))
    assert min(len(a) + len(b) for a, b in pairs) >= 8192
    ctx = pg.Context(0)
    cm = pg.CostMatrix.of_list(ctx, STD_TCM, 0)
    ctx.set_speculation(0)
    ref = pg.median_batch(ctx, cm, pairs)
    assert np.all(ref.status == 0)
    dref = pg.distance_batch(ctx, cm, pairs)
    ocm = oracle.cm(tcm=STD_TCM)
    for k in (0, 7, 13):
        r = oracle.median(ocm, *pairs[k], False)
        assert ref.cost[k] == r.cost and np.array_equal(ref.pair(k).aligned_a, r.ea), k
    for passes in (1, 2, 4, 8):
        ctx.set_speculation(1, passes)
        _same(ref, pg.median_batch(ctx, cm, pairs))
        d = pg.distance_batch(ctx, cm, pairs)
        assert np.array_equal(d[0], dref[0]) and np.array_equal(d[1], dref[1])
    ctx.close()
