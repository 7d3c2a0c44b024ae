"""Cost-only scoring (SeqCS.DOS.distance): algn_CAML_cost_affine_3's full
unbanded affine fill and the linear cost_2 with deltaw = max 8 |la - lb|,
against the oracle (itself pinned to the reference build)."""
import numpy as np
import pytest

from cases import AFF_TCM, STD_TCM, edge_pairs, mutate, random_pairs, rseq
from poy5_gb300 import workloads as wl

GAP = 16


def _count_gaps(s):
    s = np.asarray(s)
    return int(np.count_nonzero((s >= GAP) & ((s & GAP) != 0)))


def oracle_distance(oracle, ocm, a, b, affine, missing):
    """DOS.distance restated over the oracle's entry points."""
    if np.all(np.asarray(a) == GAP) or np.all(np.asarray(b) == GAP):
        return missing
    if affine:
        return oracle.cost_affine(ocm, a, b)
    la, lb = len(a), len(b)
    deltaw = max(8, abs(la - lb))
    s1, s2 = (a, b) if la <= lb else (b, a)
    lower = int(len(s1) * 0.10)
    dw = lower if len(s1) - len(s2) < lower else deltaw
    return oracle.simple_2(ocm, s1, s2, max(_count_gaps(a), _count_gaps(b)) + dw)


def test_oracle_distance_missing(oracle):
    ocm = oracle.cm(tcm=STD_TCM)
    g = np.array([GAP, GAP, GAP], np.uint8)
    assert oracle_distance(oracle, ocm, g, rseq(np.random.default_rng(1), 9), False, 77) == 77


def _cases(rng, n, maxlen):
    pairs = edge_pairs() + random_pairs(rng, n, maxlen=maxlen)
    # tiny sequences, all-gap sequences, equal lengths
    pairs += [(np.array([GAP], np.uint8), rseq(rng, 5)), (rseq(rng, 1), rseq(rng, 1)),
              (rseq(rng, 0), rseq(rng, 1)), (rseq(rng, 1), rseq(rng, 2)),
              (rseq(rng, 2), rseq(rng, 2)), (rseq(rng, 3), rseq(rng, 2)),
              (rseq(rng, 2), rseq(rng, 7)), (np.array([GAP, GAP, GAP], np.uint8), rseq(rng, 30))]
    pairs += [(rseq(rng, int(rng.integers(1, 4)), gapp=0.3), rseq(rng, int(rng.integers(1, 4))))
              for _ in range(20)]
    s = rseq(rng, 40)
    pairs.append((s, s.copy()))
    return pairs


@pytest.mark.gpu
def test_cost_affine_3_matches_oracle(ctx, oracle):
    import poy5_gb300 as pg
    cm = pg.CostMatrix.of_list(ctx, AFF_TCM, 3)
    ocm = oracle.cm(tcm=AFF_TCM, gap_open=3)
    al = pg.Align(ctx)
    rng = np.random.default_rng(31)
    for a, b in _cases(rng, 150, 400):
        for x, y in ((a, b), (b, a)):
            assert al.cost_affine_3(x, y, cm) == oracle.cost_affine(ocm, x, y), (len(x), len(y))


@pytest.mark.gpu
@pytest.mark.parametrize("affine", [False, True])
def test_distance_batch_matches_oracle(ctx, oracle, affine):
    import poy5_gb300 as pg
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    ocm = oracle.cm(tcm=tcm, gap_open=go)
    rng = np.random.default_rng(41 + affine)
    pairs = _cases(rng, 500, 1200)
    cost, status = pg.distance_batch(ctx, cm, pairs, missing_distance=12345)
    for k, (a, b) in enumerate(pairs):
        assert status[k] == 0, (k, status[k])
        assert cost[k] == oracle_distance(oracle, ocm, a, b, affine, 12345), (k, len(a), len(b))


@pytest.mark.gpu
def test_distance_batch_serving_sample(ctx, oracle):
    """Long, 30%-divergent pairs of the serving workload (up to 5,000)."""
    import poy5_gb300 as pg
    w = wl.serving_pairs(n_pairs=48, seed=wl.SEED_BASE + 40)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ocm = oracle.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    cost, status = pg.distance_batch(ctx, cm, w.pairs)
    assert np.all(status == 0)
    for k, (a, b) in enumerate(w.pairs):
        assert cost[k] == oracle.cost_affine(ocm, a, b), k


@pytest.mark.gpu
def test_distance_batch_long_prefix_matches_oracle(ctx, oracle):
    """A batch large enough for one pair per warp whose longest pairs (at
    least 2^22 cells) go one per CTA: column-block counts of every residue
    modulo the CTA's warps, unequal lengths, a long all-gap sequence."""
    import poy5_gb300 as pg
    cm = pg.CostMatrix.of_list(ctx, AFF_TCM, 3)
    ocm = oracle.cm(tcm=AFF_TCM, gap_open=3)
    rng = np.random.default_rng(47)
    pairs = random_pairs(rng, 420, maxlen=300)
    for la, lb in ((2100, 2100), (2400, 2050), (2050, 2600), (2900, 2300), (3300, 2100),
                   (2200, 4000)):
        a = rseq(rng, la - 1)
        b = np.asarray(mutate(rng, a, 0.2, 0.03), np.uint8)
        b = b[:lb] if len(b) >= lb else np.concatenate([b, rseq(rng, lb - len(b))[1:]])
        pairs.append((a, b))
    pairs.append((np.full(2100, GAP, np.uint8), rseq(rng, 2100)))
    order = rng.permutation(len(pairs))
    pairs = [pairs[k] for k in order]
    assert len(pairs) > 2 * 152
    cost, status = pg.distance_batch(ctx, cm, pairs, missing_distance=999)
    for k, (a, b) in enumerate(pairs):
        assert status[k] == 0, (k, status[k])
        assert cost[k] == oracle_distance(oracle, ocm, a, b, True, 999), (k, len(a), len(b))
