"""Every pair of the two batch workloads, bit-exact against the oracle.

The plain pairwise workload (4,096 linear pairs, lengths 200-600, 1 %
ambiguity codes, subs 1 / indel 2) and the affine pair workload (65,536
pairs, lognormal lengths with median 800, gap opening 3, extension 1,
subs 1) at their full sizes: cost, worst cost, aligned pair, median and
median with gaps of each pair, byte for byte, against the oracle's C
restatement run over the same pairs on all host cores.
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
