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


def test_long_pairs_full_length_match_oracle(ctx, oracle):
    """Six pairs of the long-pair workload at full length (both sequences
    40-49 kb): the widest band classes and the 64-bit direction indices,
    where the reference's own int index products (src/algn.c:985, 1019,
    3287) would pass 2^31; the oracle indexes in 64 bits."""
    import poy5_gb300 as pg
    from oracle_lib import compare_batch
    w = wl.long_pairs(n_pairs=16, seed=wl.SEED_BASE + 51)
    pairs = [(a, b) for a, b in w.pairs if min(len(a), len(b)) >= 40000]
    assert len(pairs) >= 4
    assert max(len(a) * len(b) for a, b in pairs) >= 2 ** 31
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ocm = oracle.cm(subs=w.subs, indel=w.indel)
    pk = pg.pack_pairs(pairs)
    res = pg.median_batch(ctx, cm, pk)
    assert np.all(res.status == 0), res.status
    ref = oracle.median_batch(ocm, [a for a, _ in pairs], [b for _, b in pairs], False,
                              len(pairs))
    ints = [res.cost, res.maxcost, res.alen, res.mlen, res.wlen, res.status]
    par = compare_batch(ref, ints, [res.ea, res.eb, res.med, res.mwg], pk.out_off, pk.cap)
    assert par["mismatches"] == 0, par
