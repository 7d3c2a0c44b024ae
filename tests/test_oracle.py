"""The oracle (C restatement) pinned to the reference POY algn.c.

* against the golden fixtures generated from the reference build (always);
* against the reference build itself on fresh random inputs, when the
  reference library was built on this machine (oracle/_ref).
"""
import numpy as np
import pytest

import golden_lib
from cases import AFF_TCM, STD_TCM, edge_pairs, random_pairs
from oracle_lib import Oracle, available


@pytest.mark.parametrize("name", golden_lib.NAMES)
def test_oracle_matches_golden(oracle, name):
    g = golden_lib.load(name)
    cm = oracle.cm(tcm=g.tcm.tolist(), gap_open=g.gap_open)
    t = oracle.tables(cm)
    for key, want in g.tables.items():
        assert np.array_equal(t[key], want), key
    oracle.set_check(True)
    for k, (a, b) in enumerate(g.pairs):
        r = oracle.median(cm, a, b, g.affine)
        bad = golden_lib.mismatches(g, k, r.cost, r.ea, r.eb, r.median, r.medianwg, r.maxcost)
        assert not bad, (name, k, bad)


def test_hand_checked_costs(oracle):
    """Costs derivable by hand from the DP definition (subs 1, indel 2)."""
    cm = oracle.cm(tcm=STD_TCM)
    enc = {"A": 1, "C": 2, "G": 4, "T": 8, "R": 5}
    S = lambda t: np.array([16] + [enc[c] for c in t], np.uint8)
    assert oracle.median(cm, S("ACGT"), S("ACGT"), False).cost == 0
    assert oracle.median(cm, S("ACGT"), S("AGGT"), False).cost == 1
    assert oracle.median(cm, S("ACGT"), S("AGT"), False).cost == 2
    r = oracle.median(cm, S("A"), S("R"), False)  # A vs A|G
    assert r.cost == 0 and list(r.median) == [16, 1]


needs_ref = pytest.mark.skipif(not available("ref"), reason="reference build absent")


@needs_ref
@pytest.mark.parametrize("affine", [False, True])
def test_oracle_matches_reference_random(affine):
    port, ref = Oracle("port"), Oracle("ref")
    port.set_check(True)
    rng = np.random.default_rng(99 + affine)
    tcm = AFF_TCM if affine else STD_TCM
    go = 3 if affine else 0
    cp, cr = port.cm(tcm=tcm, gap_open=go), ref.cm(tcm=tcm, gap_open=go)
    for a, b in edge_pairs() + random_pairs(rng, 400, maxlen=500):
        x, y = port.median(cp, a, b, affine), ref.median(cr, a, b, affine)
        assert x.cost == y.cost and x.maxcost == y.maxcost
        for f in ("ea", "eb", "median", "medianwg"):
            assert np.array_equal(getattr(x, f), getattr(y, f)), f


@needs_ref
def test_oracle_matches_reference_random_tcm():
    port, ref = Oracle("port"), Oracle("ref")
    rng = np.random.default_rng(5)
    for t in range(40):
        M = rng.integers(1, 6, (5, 5))
        if t % 3:
            M = np.triu(M) + np.triu(M, 1).T
        if t % 4:
            np.fill_diagonal(M, 0)
        go = int(rng.integers(0, 4))
        cp, cr = port.cm(tcm=M.tolist(), gap_open=go), ref.cm(tcm=M.tolist(), gap_open=go)
        tp, tr = port.tables(cp), ref.tables(cr)
        for key in ("cost", "median", "worst", "tail", "prepend"):
            assert np.array_equal(tp[key], tr[key]), (t, key)
        for a, b in random_pairs(rng, 6, maxlen=200):
            x, y = port.median(cp, a, b, go > 0), ref.median(cr, a, b, go > 0)
            assert (x.cost, x.maxcost) == (y.cost, y.maxcost)
            assert np.array_equal(x.median, y.median)


@needs_ref
def test_oracle_stubs_match_reference():
    """Raw algn_CAML_simple_2 / backtrace_2d, including the full-plane branch
    (large deltawh) and both tie preferences; cost-only affine."""
    port, ref = Oracle("port"), Oracle("ref")
    rng = np.random.default_rng(11)
    cp, cr = port.cm(tcm=STD_TCM), ref.cm(tcm=STD_TCM)
    ap, ar = port.cm(tcm=AFF_TCM, gap_open=3), ref.cm(tcm=AFF_TCM, gap_open=3)
    # algn_CAML_cost_affine_3 carves 12 rows of max(len) ints out of a
    # (max(len)+1)^2 workspace: below length 11 it writes past the
    # allocation unless an earlier call already grew the shared workspace.
    # Grow it once, as any real POY session has.
    big = np.concatenate([[16], rng.choice(np.array([1, 2, 4, 8], np.uint8), 64)]).astype(np.uint8)
    ref.cost_affine(ar, big, big)
    for a, b in random_pairs(rng, 60, maxlen=300):
        s1, s2 = (a, b) if len(a) <= len(b) else (b, a)
        for dwh in (0, 3, 40, 400):
            assert port.simple_2(cp, s1, s2, dwh) == ref.simple_2(cr, s1, s2, dwh)
            for sw in (0, 1):
                x, y = port.backtrace_2d(cp, s1, s2, sw), ref.backtrace_2d(cr, s1, s2, sw)
                assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
        assert port.cost_affine(ap, a, b) == ref.cost_affine(ar, a, b)
        for dw in (-1, 8):
            assert port.cost_linear(cp, a, b, dw) == ref.cost_linear(cr, a, b, dw)


def test_schedule_cells_match_oracle(oracle):
    """Host schedule arithmetic (used for GCUPS) vs the oracle's own count."""
    from poy5_gb300 import schedule
    rng = np.random.default_rng(3)
    for affine in (False, True):
        tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
        cm = oracle.cm(tcm=tcm, gap_open=go)
        pairs = random_pairs(rng, 150, maxlen=600)
        la = np.array([len(a) for a, _ in pairs])
        lb = np.array([len(b) for _, b in pairs])
        its, want = zip(*[oracle.schedule(cm, a, b, affine) for a, b in pairs])
        full = None
        if not affine:
            g = lambda s: int(np.count_nonzero((s >= 16) & ((s & 16) != 0)))
            full = schedule.linear_full_plane(la, lb, [g(a) for a, _ in pairs],
                                              [g(b) for _, b in pairs])
            # the oracle reports 0 iterations for a full plane
            assert all((i == 0) == f for i, f in zip(its, full))
        got = schedule.cells_computed(la, lb, np.array(its), 1, affine, full)
        ok = [a > 1 or affine is False for a in np.minimum(la, lb)]
        assert np.array_equal(got[ok], np.array(want)[ok])


def test_schedule_skipped_passes_accounting():
    """cells_computed with skipped leading passes: the full schedule's cells
    minus those of the skipped passes (every pair skipping some)."""
    from poy5_gb300 import schedule
    rng = np.random.default_rng(5)
    la = rng.integers(2, 3000, 500)
    lb = (la + rng.integers(0, 40, 500)).astype(np.int64)
    for affine in (False, True):
        s = schedule.unstoppable_passes(la, lb, 1, affine)
        assert s.min() >= 1
        passes = s + rng.integers(1, 4, 500)
        full = schedule.cells_computed(la, lb, passes, 1, affine)
        head = schedule.cells_computed(la, lb, s, 1, affine)
        got = schedule.cells_computed(la, lb, passes, 1, affine, skipped=s)
        assert np.array_equal(got, full - head)
