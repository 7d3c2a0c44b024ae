"""GPU parity: libpoyalgn.so against the reference (golden fixtures) and the
oracle, bit-exact on cost, aligned pair, medians and worst cost.
"""
import numpy as np
import pytest

import golden_lib
from cases import AFF_TCM, STD_TCM, edge_pairs, random_pairs

pytestmark = pytest.mark.gpu


def _cm(ctx, tcm, go):
    import poy5_gb300 as pg
    return pg.CostMatrix.of_list(ctx, tcm, go)


@pytest.mark.parametrize("name", golden_lib.NAMES)
def test_batch_matches_golden(ctx, name):
    import poy5_gb300 as pg
    g = golden_lib.load(name)
    cm = _cm(ctx, g.tcm, g.gap_open)
    t = cm.tables()
    for key, want in g.tables.items():
        assert np.array_equal(t[key], want), key
    res = pg.median_batch(ctx, cm, g.pairs)
    assert np.all(res.status == 0), res.status
    for k in range(len(g.pairs)):
        d = res.pair(k)
        bad = golden_lib.mismatches(g, k, d.cost, d.aligned_a, d.aligned_b, d.median,
                                    d.median_wg, d.maxcost)
        assert not bad, (name, k, bad)


@pytest.mark.parametrize("affine", [False, True])
def test_batch_matches_oracle_random(ctx, oracle, affine):
    import poy5_gb300 as pg
    rng = np.random.default_rng(2024 + affine)
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    cm = _cm(ctx, tcm, go)
    ocm = oracle.cm(tcm=tcm, gap_open=go)
    pairs = edge_pairs() + random_pairs(rng, 600, maxlen=900)
    res = pg.median_batch(ctx, cm, pairs)
    for k, (a, b) in enumerate(pairs):
        try:
            r = oracle.median(ocm, a, b, affine)
        except Exception as e:
            # an empty affine median is undefined in POY (it reads median[0]
            # of an empty sequence); both sides must refuse the pair
            assert "empty" in str(e) and res.status[k] == -4, (k, res.status[k], e)
            continue
        assert res.status[k] == 0, (k, res.status[k])
        d = res.pair(k)
        assert (d.cost, d.maxcost) == (r.cost, r.maxcost), k
        assert np.array_equal(d.aligned_a, r.ea) and np.array_equal(d.aligned_b, r.eb), k
        assert np.array_equal(d.median, r.median), k
        assert np.array_equal(d.median_wg, r.medianwg), k


def test_batch_workload_samples(ctx, oracle):
    """Slices of the two benchmark workloads, against the oracle."""
    import poy5_gb300 as pg
    from poy5_gb300 import workloads as wl
    for w in (wl.plain_pairs(n_pairs=96), wl.affine_pairs(n_pairs=192)):
        cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
        ocm = oracle.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
        res = pg.median_batch(ctx, cm, w.pairs)
        assert np.all(res.status == 0)
        out = oracle.median_batch(ocm, [a for a, _ in w.pairs], [b for _, b in w.pairs],
                                  w.affine)
        assert np.array_equal(res.cost, out["cost"])
        assert np.array_equal(res.maxcost, out["maxcost"])
        for k in range(len(w.pairs)):
            o = int(out["out_off"][k])
            d = res.pair(k)
            assert np.array_equal(d.median, out["med"][o:o + out["mlen"][k]])
            assert np.array_equal(d.aligned_a, out["ea"][o:o + out["alen"][k]])


def test_per_call_stubs_match_oracle(ctx, oracle):
    """simple_2 + backtrace_2d, align_affine_3, aligned medians, dos_median."""
    import poy5_gb300 as pg
    rng = np.random.default_rng(77)
    cm, acm = _cm(ctx, STD_TCM, 0), _cm(ctx, AFF_TCM, 3)
    ocm, oacm = oracle.cm(tcm=STD_TCM), oracle.cm(tcm=AFF_TCM, gap_open=3)
    al = pg.Align(ctx)
    for a, b in edge_pairs()[:8] + random_pairs(rng, 40, maxlen=300):
        s1, s2 = (a, b) if len(a) <= len(b) else (b, a)
        for dwh in (0, 40, 400):
            assert al.c_cost_2(s1, s2, cm, dwh) == oracle.simple_2(ocm, s1, s2, dwh)
            for sw in (0, 1):
                x = al.extract_edited_2(s1, s2, cm, sw)
                y = oracle.backtrace_2d(ocm, s1, s2, sw)
                assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
        for cmx, ocmx, aff in ((cm, ocm, False), (acm, oacm, True)):
            d = pg.dos_median(al, a, b, cmx)
            r = oracle.median(ocmx, a, b, aff)
            assert (d.cost, d.maxcost) == (r.cost, r.maxcost)
            assert np.array_equal(d.median, r.median)
            assert np.array_equal(d.median_wg, r.medianwg)
            assert np.array_equal(d.aligned_a, r.ea) and np.array_equal(d.aligned_b, r.eb)


def test_errors_are_loud(ctx):
    import poy5_gb300 as pg
    al = pg.Align(ctx)
    cm = _cm(ctx, AFF_TCM, 3)
    long_, short = pg.encode("ACGTACGT"), pg.encode("ACG")
    with pytest.raises(pg.PoyAlgnError):
        al.c_align_affine_3(long_, short, cm, 0)  # "pass the shorter one as first"
    with pytest.raises(pg.PoyAlgnError):
        al.extract_edited_2(pg.encode("AC"), pg.encode("ACGA"), _cm(ctx, STD_TCM, 0), 0)


@pytest.mark.parametrize("name", golden_lib.NAMES)
def test_adopted_reference_tables_match_golden(ctx, name):
    """poyalgn_cm_adopt, the route the POY stub library takes a struct cm by:
    the reference's own tables from the golden file (as cm_CAML_create and
    the OCaml setters left them: lcm 5, gap 16, 31 states with combinations)
    give the golden results."""
    import poy5_gb300 as pg
    g = golden_lib.load(name)
    t = g.tables
    cm = pg.CostMatrix.adopt(ctx, 5, 16, 31, 1, 1 if g.affine else 0, g.gap_open,
                             t["cost"], t["median"], t["worst"], t["tail"], t["prepend"])
    back = cm.tables()
    for key, want in t.items():
        assert np.array_equal(back[key], want), key
    res = pg.median_batch(ctx, cm, g.pairs)
    assert np.all(res.status == 0), res.status
    for k in range(len(g.pairs)):
        d = res.pair(k)
        bad = golden_lib.mismatches(g, k, d.cost, d.aligned_a, d.aligned_b, d.median,
                                    d.median_wg, d.maxcost)
        assert not bad, (name, k, bad)
