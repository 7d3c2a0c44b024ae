"""Tree downpass over device-resident sequences: host logic on the CPU, and
on the GPU the per-node medians and total tree cost against the oracle's
node-by-node DOS.median recursion."""
import numpy as np
import pytest

from poy5_gb300 import workloads as wl
from poy5_gb300.tree import tree_levels


def _oracle_downpass(oracle, ocm, t):
    seqs = list(t.leaves)
    costs = []
    for a, b in zip(t.left, t.right):
        r = oracle.median(ocm, seqs[a], seqs[b], t.affine)
        seqs.append(r.median)
        costs.append(r.cost)
    return seqs[len(t.leaves):], np.array(costs)


def test_yule_tree_shape():
    t = wl.yule_tree(n_taxa=64, root_len=200)
    n = len(t.leaves)
    assert n == 64 and len(t.left) == n - 1
    used = np.concatenate([t.left, t.right])
    # every node but the root is a child exactly once
    assert sorted(used.tolist()) == list(range(2 * n - 2))
    assert all(s[0] == wl.GAP and np.all(s[1:] < wl.GAP) for s in t.leaves)
    lv = tree_levels(n, t.left, t.right)
    assert lv[-1] == lv.max() and lv.min() == 1


def test_tree_levels_rejects_forward_children():
    with pytest.raises(ValueError):
        tree_levels(2, [0, 3], [1, 2])


def test_oracle_downpass_small(oracle):
    t = wl.yule_tree(n_taxa=8, root_len=60)
    ocm = oracle.cm(subs=t.subs, indel=t.indel)
    meds, costs = _oracle_downpass(oracle, ocm, t)
    assert len(meds) == 7 and costs.sum() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("n_taxa,root_len", [(16, 120), (256, 1500)])
def test_downpass_matches_oracle(ctx, oracle, n_taxa, root_len):
    import poy5_gb300 as pg
    t = wl.yule_tree(n_taxa=n_taxa, root_len=root_len)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, t.subs, t.indel, t.gap_open)
    ocm = oracle.cm(subs=t.subs, indel=t.indel)
    store = pg.Store(ctx, 64 << 20)
    leaf_nodes = [store.add(s) for s in t.leaves]
    res = pg.downpass(store, cm, leaf_nodes, t.left, t.right)
    meds, costs = _oracle_downpass(oracle, ocm, t)
    assert np.array_equal(res.internal_cost, costs)
    assert res.total_cost == int(costs.sum())
    assert res.levels == int(tree_levels(n_taxa, t.left, t.right).max())
    for k, m in enumerate(meds):
        assert np.array_equal(store.read(int(res.internal_node[k])), m), k


@pytest.mark.gpu
def test_store_batch_matches_host_batch(ctx):
    import poy5_gb300 as pg
    w = wl.affine_pairs(n_pairs=64)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    store = pg.Store(ctx, 16 << 20)
    na = [store.add(a) for a, _ in w.pairs]
    nb = [store.add(b) for _, b in w.pairs]
    ref = pg.median_batch(ctx, cm, w.pairs)
    n0 = len(store)
    med, cost, mx, st = store.median_batch(cm, na, nb, keep=False)
    assert len(store) == n0 and np.all(st == 0) and np.all(med == -1)
    assert np.array_equal(cost, ref.cost) and np.array_equal(mx, ref.maxcost)
    med, cost, mx, st = store.median_batch(cm, na, nb, keep=True)
    assert np.array_equal(cost, ref.cost)
    for k in range(len(w.pairs)):
        assert np.array_equal(store.read(int(med[k])), ref.pair(k).median), k
    store.truncate(n0)
    assert len(store) == n0


# ---- uppass: SeqCS.DOS.median_3_no_union, top down -----------------------------

def _median2_no_gaps(tab, ea, eb):
    """seq_get_median_2d_no_gaps (src/seq.c:259-272) on an aligned pair."""
    med, lcm, gap = tab["median"], tab["lcm"], tab["gap"]
    out = [int(med[(int(x) << lcm) + int(y)]) for x, y in zip(ea, eb)]
    return np.array([gap] + [v for v in out if v != gap], np.uint8)


def _oracle_median3(oracle, ocm, tab, p, c1, c2, affine):
    """SeqCS.DOS.median_3_no_union (src/seqCS.ml:1123-1147) over the oracle's
    Align.align_2 (parent first): the cheaper alignment, the second on a tie."""
    r1 = oracle.median(ocm, p, c1, affine)
    r2 = oracle.median(ocm, p, c2, affine)
    r = r1 if r1.cost < r2.cost else r2
    return _median2_no_gaps(tab, r.ea, r.eb), r.cost, r.maxcost


def _oracle_uppass(oracle, ocm, t, prelim):
    """Root keeps its downpass state; every other internal node takes
    median_3_no_union(parent final, children states)."""
    tab = oracle.tables(ocm)
    nl, ni = len(t.leaves), len(t.left)
    state = lambda ch: t.leaves[ch] if ch < nl else prelim[ch - nl]
    parent = {}
    for k in range(ni):
        for ch in (t.left[k], t.right[k]):
            if ch >= nl:
                parent[ch - nl] = k
    final, cost = [None] * ni, [0] * ni
    final[ni - 1] = prelim[ni - 1]
    for k in range(ni - 2, -1, -1):  # parents come after their children
        final[k], cost[k], _ = _oracle_median3(oracle, ocm, tab, final[parent[k]],
                                               state(t.left[k]), state(t.right[k]), t.affine)
    return final, np.array(cost)


def test_oracle_uppass_small(oracle):
    t = wl.yule_tree(n_taxa=8, root_len=60)
    ocm = oracle.cm(subs=t.subs, indel=t.indel)
    meds, _ = _oracle_downpass(oracle, ocm, t)
    final, cost = _oracle_uppass(oracle, ocm, t, meds)
    assert len(final) == 7 and all(f[0] == wl.GAP for f in final) and cost[-1] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("n_taxa,root_len", [(16, 120), (64, 600)])
def test_uppass_matches_oracle(ctx, oracle, n_taxa, root_len):
    import poy5_gb300 as pg
    t = wl.yule_tree(n_taxa=n_taxa, root_len=root_len)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, t.subs, t.indel, t.gap_open)
    ocm = oracle.cm(subs=t.subs, indel=t.indel)
    store = pg.Store(ctx, 64 << 20)
    leaf_nodes = [store.add(s) for s in t.leaves]
    down = pg.downpass(store, cm, leaf_nodes, t.left, t.right)
    up = pg.uppass(store, cm, leaf_nodes, t.left, t.right, down.internal_node)
    meds, _ = _oracle_downpass(oracle, ocm, t)
    final, cost = _oracle_uppass(oracle, ocm, t, meds)
    assert np.array_equal(up.final_cost, cost)
    assert up.final_node[-1] == down.internal_node[-1]
    for k, f in enumerate(final):
        assert np.array_equal(store.read(int(up.final_node[k])), f), k


@pytest.mark.gpu
def test_median3_batch_affine_matches_oracle(ctx, oracle):
    """Affine triples: the no-gap median of the kept aligned pair differs from
    DOS.median's own median, so this checks the separate median path."""
    import poy5_gb300 as pg
    w = wl.affine_pairs(n_pairs=48, seed=wl.SEED_BASE + 70)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ocm = oracle.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    tab = oracle.tables(ocm)
    store = pg.Store(ctx, 32 << 20)
    rng = np.random.default_rng(71)
    # related triples: a parent, its workload partner, and a third variant
    seqs = []
    for a, b in w.pairs[:40]:
        c = wl.with_gap(wl.mutate(rng, a[1:], 0.1, 0.02))
        seqs.append((a, b, c if len(c) > 1 else b))
    ids = np.array([[store.add(s) for s in t] for t in seqs], np.int32)
    node, cost, mx, st = store.median3_batch(cm, ids[:, 0], ids[:, 1], ids[:, 2])
    assert np.all(st == 0), st
    for k, (p, a, b) in enumerate(seqs):
        m, c, x = _oracle_median3(oracle, ocm, tab, p, a, b, True)
        assert (cost[k], mx[k]) == (c, x), k
        assert np.array_equal(store.read(int(node[k])), m), k


# ---- Align.closest --------------------------------------------------------------

def _closest_state(tab, a, b):
    """Cost_matrix.Two_D.get_closest (src/cost_matrix.ml:1387-1426), with
    combinations and no levels."""
    gap, lcm = tab["gap"], tab["lcm"]
    bb = b if (a == gap or b == gap) else (gap if (a & gap and b & gap) else b & ~gap)
    best, bc = 0, None
    for bit in range(lcm):
        x = 1 << bit
        if bb & x:
            c = int(tab["cost"][(a << lcm) + x])
            if bc is None or c < bc:
                best, bc = x, c
    return best


def _oracle_closest(oracle, ocm, tab, s1, s2, affine):
    """Sequence.Align.closest (src/sequence.ml:1180-1237) over the oracle."""
    gap = tab["gap"]
    if np.all(s2 == gap):
        return s2, 0
    if len(s1) == len(s2) and np.array_equal(s1, s2):
        a, b = s1.astype(int), s2.astype(int)
        a[1:] &= ~gap
        b[1:] &= ~gap
        comp = True
    else:
        r = oracle.median(ocm, s1, s2, affine)
        a, b, comp = r.ea.astype(int), r.eb.astype(int), False
    out = [_closest_state(tab, int(x), int(y)) for x, y in zip(a, b)]
    res = np.array([gap] + [v for v in out if v != gap], np.uint8)
    if comp:
        return res, 0
    return res, (oracle.cost_affine(ocm, s1, res) if affine else oracle.cost_linear(ocm, s1, res))


@pytest.mark.gpu
@pytest.mark.parametrize("affine", [False, True])
def test_closest_batch_matches_oracle(ctx, oracle, affine):
    import poy5_gb300 as pg
    from cases import AFF_TCM, STD_TCM, random_pairs, rseq
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    ocm = oracle.cm(tcm=tcm, gap_open=go)
    tab = oracle.tables(ocm)
    rng = np.random.default_rng(81 + affine)
    # ambiguous and gap-bearing states, an all-gap second sequence, equal pairs
    pairs = [(a, b) for a, b in random_pairs(rng, 60, maxlen=500, kinds=3)]
    s = rseq(rng, 50, amb=0.2)
    pairs += [(s, s.copy()), (rseq(rng, 30), np.full(4, wl.GAP, np.uint8))]
    store = pg.Store(ctx, 16 << 20)
    n1 = [store.add(a) for a, _ in pairs]
    n2 = [store.add(b) for _, b in pairs]
    node, cost, st = store.closest_batch(cm, n1, n2)
    for k, (a, b) in enumerate(pairs):
        try:
            want, c = _oracle_closest(oracle, ocm, tab, a, b, affine)
        except Exception:
            continue  # the reference fails (empty state); the status says so
        assert st[k] == 0, (k, st[k])
        assert cost[k] == c, k
        assert np.array_equal(store.read(int(node[k])), want), k


# ---- Sequence.readjust ----------------------------------------------------------

def _oracle_readjust(oracle, ocm, tab, a, b, c, affine):
    """Sequence.readjust (src/sequence.ml:2097-2158) over the oracle: algn is
    DOS.median's (cost, median)."""
    def algn(x, y):
        r = oracle.median(ocm, x, y, affine)
        return r.cost, r.median
    cab, ab = algn(a, b)
    cbc, bc = algn(b, c)
    cac, ac = algn(a, c)
    cabc = algn(ab, c)[0] + cab
    cbca = algn(bc, a)[0] + cbc
    cacb = algn(ac, b)[0] + cac
    if cabc <= cbca:
        p, q = (c, ab) if cabc <= cacb else (b, ac)
    elif cbca < cacb:
        p, q = a, bc
    else:
        p, q = b, ac
    m, _ = _oracle_closest(oracle, ocm, tab, p, q, affine)
    cost2 = algn(a, m)[0] + algn(b, m)[0]
    return m, cost2 + algn(c, m)[0], cost2


@pytest.mark.gpu
@pytest.mark.parametrize("affine", [False, True])
def test_readjust_batch_matches_oracle(ctx, oracle, affine):
    import poy5_gb300 as pg
    from cases import AFF_TCM, STD_TCM
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    ocm = oracle.cm(tcm=tcm, gap_open=go)
    tab = oracle.tables(ocm)
    rng = np.random.default_rng(91 + affine)
    trip = []
    for _ in range(24):  # a node's two children and its parent, related
        root = wl.random_bases(rng, int(rng.integers(40, 400)))
        trip.append(tuple(wl.with_gap(wl.mutate(rng, root, 0.1, 0.03)) for _ in range(3)))
    store = pg.Store(ctx, 16 << 20)
    ids = np.array([[store.add(s) for s in t] for t in trip], np.int32)
    node, c3, c2, st = store.readjust_batch(cm, ids[:, 0], ids[:, 1], ids[:, 2])
    assert np.all(st == 0), st
    for k, (a, b, c) in enumerate(trip):
        m, w3, w2 = _oracle_readjust(oracle, ocm, tab, a, b, c, affine)
        assert (c3[k], c2[k]) == (w3, w2), k
        assert np.array_equal(store.read(int(node[k])), m), k
