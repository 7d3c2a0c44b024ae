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
    its backtrace asserts (src/newkkonen.c:786-790, 1554): only affine."""
    cm = oracle.cm(subs=1, indel=2)
    with pytest.raises(OracleError):
        oracle.newkk_median(cm, np.array([16, 1], np.uint8), np.array([16, 2], np.uint8))
