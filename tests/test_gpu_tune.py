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
