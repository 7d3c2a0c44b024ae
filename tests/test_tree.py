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
