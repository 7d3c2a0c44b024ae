"""Every pair of the two batch workloads, bit-exact against the oracle.

The plain pairwise workload (4,096 linear pairs, lengths 200-600, 1 %
ambiguity codes, subs 1 / indel 2) and the affine pair workload (65,536
pairs, lognormal lengths with median 800, gap opening 3, extension 1,
subs 1) at their full sizes: cost, worst cost, aligned pair, median and
median with gaps of each pair, byte for byte, against the oracle's C
restatement run over the same pairs on all host cores. The three-sequence
workload (8,192 readjust triples) likewise: cost, length and the three
aligned sequences of every triple.
"""
import os

import pytest

from poy5_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["plain_pairs", "affine_pairs"])
def test_full_workload_matches_oracle(ctx, oracle, name):
    import poy5_gb300 as pg
    from oracle_lib import compare_batch
    w = wl.plain_pairs() if name == "plain_pairs" else wl.affine_pairs()
    assert len(w.pairs) == (4096 if name == "plain_pairs" else 65536)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    pk = pg.pack_pairs(w.pairs)
    res = pg.median_batch(ctx, cm, pk)
    ocm = oracle.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    ref = oracle.median_batch(ocm, [a for a, _ in w.pairs], [b for _, b in w.pairs], w.affine,
                              os.cpu_count() or 1)
    ints = [res.cost, res.maxcost, res.alen, res.mlen, res.wlen, res.status]
    par = compare_batch(ref, ints, [res.ea, res.eb, res.med, res.mwg], pk.out_off, pk.cap)
    assert par["mismatches"] == 0, par


def test_full_readjust_triples_match_oracle(ctx, oracle):
    """Every one of the 8,192 three-sequence alignments the bench times
    (readjust_triples_8192x100-300_linear): cost, length and the three
    aligned sequences against the oracle restatement on all host cores."""
    import numpy as np
    import poy5_gb300 as pg
    from poy5_gb300.three_d import pack_triples
    w = wl.readjust_triples(n_triples=8192)
    res = pg.powell_3d_batch(ctx, w.triples, w.mm, w.go, w.ge)
    seqs, off, lens, out_off, cap = pack_triples(w.triples)
    ref = oracle.powell_3d_batch(seqs, off, lens, out_off, w.mm, w.go, w.ge,
                                 nthreads=os.cpu_count() or 1)
    assert (ref["status"] == 0).all() and (res.status == 0).all()
    assert np.array_equal(ref["cost"], res.cost)
    assert np.array_equal(ref["rlen"], res.rlen)
    # the bytes each triple's alignment occupies: the rlen bytes that end at
    # its slot's end (the rest of a slot is never written)
    n = res.rlen.astype(np.int64)
    end = out_off + cap
    idx = np.repeat(end - n, n) + (np.arange(int(n.sum())) - np.repeat(np.cumsum(n) - n, n))
    for name, got in (("ra", res.ra), ("rb", res.rb), ("rc", res.rc)):
        assert np.array_equal(ref[name][idx], got[idx]), name
