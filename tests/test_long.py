"""Long pairs (the 20-50 kb stress workload): wide bands on the largest
pipelines and 64-bit slab indexing, against the oracle."""
import numpy as np
import pytest

from poy5_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_long_pairs_match_oracle(ctx, oracle):
    import poy5_gb300 as pg
    w = wl.long_pairs(n_pairs=3, seed=wl.SEED_BASE + 50)
    w.pairs = [(a[:20001], b[:20501]) for a, b in w.pairs]  # 20 kb: seconds on the oracle
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ocm = oracle.cm(subs=w.subs, indel=w.indel)
    res = pg.median_batch(ctx, cm, w.pairs)
    assert np.all(res.status == 0), res.status
    for k, (a, b) in enumerate(w.pairs):
        r = oracle.median(ocm, a, b, False)
        d = res.pair(k)
        assert (d.cost, d.maxcost) == (r.cost, r.maxcost), k
        assert np.array_equal(d.median, r.median), k
        assert np.array_equal(d.aligned_a, r.ea) and np.array_equal(d.aligned_b, r.eb), k
