"""Pipeline ladders: results must not depend on the ladder, and the
autotuner keeps the fastest candidate."""
import numpy as np
import pytest

from poy5_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a.status, b.status)
    ok = a.status == 0
    for f in ("cost", "maxcost", "alen", "mlen", "wlen"):
        assert np.array_equal(getattr(a, f)[ok], getattr(b, f)[ok]), f
    for k in np.flatnonzero(ok):
        x, y = a.pair(k), b.pair(k)
        assert np.array_equal(x.median, y.median) and np.array_equal(x.aligned_a, y.aligned_a)
        assert np.array_equal(x.aligned_b, y.aligned_b) and np.array_equal(x.median_wg, y.median_wg)


@pytest.mark.parametrize("workload", ["affine", "linear"])
def test_every_candidate_ladder_gives_the_same_results(workload):
    import poy5_gb300 as pg
    from poy5_gb300 import tune
    w = wl.affine_pairs(n_pairs=384) if workload == "affine" else wl.plain_pairs(n_pairs=384)
    ctx = pg.Context(0)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ref = pg.median_batch(ctx, cm, w.pairs)
    assert np.all(ref.status == 0)
    for P, R in tune.candidate_ladders(w.affine)[1:]:
        tune.set_ladder(ctx, w.affine, P, R)
        assert tune.get_ladder(ctx, w.affine) == (P, R)
        _same(ref, pg.median_batch(ctx, cm, w.pairs))
    r = tune.autotune(ctx, cm, w.pairs, reps=1)
    assert tune.get_ladder(ctx, w.affine) == tuple(r["ladder"])
    assert len(r["ms"]) == len(tune.candidate_ladders(w.affine)) and min(r["ms"]) > 0
    _same(ref, pg.median_batch(ctx, cm, w.pairs))
    with pytest.raises(pg.PoyAlgnError):
        tune.set_ladder(ctx, w.affine, [4] * 10, [3] * 10)
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_lean_paths_match_oracle(oracle, mode):
    """Gap-free affine pairs on the lane pipeline (0) and on the row tile (1)."""
    import poy5_gb300 as pg
    from cases import random_pairs
    ctx = pg.Context(0)
    ctx.set_row_tile(mode)
    w = wl.affine_pairs(n_pairs=160, seed=wl.SEED_BASE + 60)
    rng = np.random.default_rng(61)
    pairs = w.pairs + [(a, b) for a, b in random_pairs(rng, 200, maxlen=700, kinds=1)]
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ocm = oracle.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    res = pg.median_batch(ctx, cm, pairs)
    for k, (a, b) in enumerate(pairs):
        try:
            r = oracle.median(ocm, a, b, True)
        except Exception as e:
            assert "empty" in str(e) and res.status[k] == -4, (k, res.status[k], e)
            continue
        assert res.status[k] == 0, (k, res.status[k])
        d = res.pair(k)
        assert (d.cost, d.maxcost) == (r.cost, r.maxcost), k
        assert np.array_equal(d.median, r.median) and np.array_equal(d.median_wg, r.medianwg), k
        assert np.array_equal(d.aligned_a, r.ea) and np.array_equal(d.aligned_b, r.eb), k
    al = pg.Align(ctx)  # per-call stubs keep a fill of either layout for the traceback
    for a, b in pairs[:12]:
        x = pg.dos_median(al, a, b, cm)
        r = oracle.median(ocm, a, b, True)
        assert x.cost == r.cost and np.array_equal(x.median, r.median)
    ctx.close()
