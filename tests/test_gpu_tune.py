"""Pipeline ladders: results must not depend on the ladder, and the
autotuner keeps the fastest candidate."""
import numpy as np
import pytest

from poy5_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a.status, b.status)
    ok = a.status == 0
    for f in ("cost", "maxcost", "alen", "mlen", "wlen"):
        assert np.array_equal(getattr(a, f)[ok], getattr(b, f)[ok]), f
    for k in np.flatnonzero(ok):
        x, y = a.pair(k), b.pair(k)
        assert np.array_equal(x.median, y.median) and np.array_equal(x.aligned_a, y.aligned_a)
        assert np.array_equal(x.aligned_b, y.aligned_b) and np.array_equal(x.median_wg, y.median_wg)


@pytest.mark.parametrize("workload", ["affine", "linear"])
def test_every_candidate_ladder_gives_the_same_results(workload):
    import poy5_gb300 as pg
    from poy5_gb300 import tune
    w = wl.affine_pairs(n_pairs=384) if workload == "affine" else wl.plain_pairs(n_pairs=384)
    ctx = pg.Context(0)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ref = pg.median_batch(ctx, cm, w.pairs)
    assert np.all(ref.status == 0)
    for P, R in tune.candidate_ladders(w.affine)[1:]:
        tune.set_ladder(ctx, w.affine, P, R)
        assert tune.get_ladder(ctx, w.affine) == (P, R)
        _same(ref, pg.median_batch(ctx, cm, w.pairs))
    r = tune.autotune(ctx, cm, w.pairs, reps=1)
    assert tune.get_ladder(ctx, w.affine) == tuple(r["ladder"])
    assert len(r["ms"]) == len(tune.candidate_ladders(w.affine)) and min(r["ms"]) > 0
    _same(ref, pg.median_batch(ctx, cm, w.pairs))
    with pytest.raises(pg.PoyAlgnError):
        tune.set_ladder(ctx, w.affine, [4] * tune.NCLASS, [5] * tune.NCLASS)
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_lean_paths_match_oracle(oracle, mode):
    """Gap-free affine pairs on the lane pipeline (0) and on the row tile (1),
    sequential passes (a speculative batch keeps the lane pipeline), the
    tracebacks deferred: through the row window for row-tile fills."""
    import poy5_gb300 as pg
    from cases import random_pairs
    ctx = pg.Context(0)
    ctx.set_row_tile(mode)
    ctx.set_speculation(0)
    w = wl.affine_pairs(n_pairs=160, seed=wl.SEED_BASE + 60)
    rng = np.random.default_rng(61)
    pairs = w.pairs + [(a, b) for a, b in random_pairs(rng, 200, maxlen=700, kinds=1)]
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    ocm = oracle.cm(subs=w.subs, indel=w.indel, gap_open=w.gap_open)
    res = pg.median_batch(ctx, cm, pairs)
    for k, (a, b) in enumerate(pairs):
        try:
            r = oracle.median(ocm, a, b, True)
        except Exception as e:
            assert "empty" in str(e) and res.status[k] == -4, (k, res.status[k], e)
            continue
        assert res.status[k] == 0, (k, res.status[k])
        d = res.pair(k)
        assert (d.cost, d.maxcost) == (r.cost, r.maxcost), k
        assert np.array_equal(d.median, r.median) and np.array_equal(d.median_wg, r.medianwg), k
        assert np.array_equal(d.aligned_a, r.ea) and np.array_equal(d.aligned_b, r.eb), k
    al = pg.Align(ctx)  # per-call stubs keep a fill of either layout for the traceback
    for a, b in pairs[:12]:
        x = pg.dos_median(al, a, b, cm)
        r = oracle.median(ocm, a, b, True)
        assert x.cost == r.cost and np.array_equal(x.median, r.median)
    ctx.close()


def test_batch_graph_replays_match_plain_calls():
    """A captured batch replayed on new contents of the same buffers."""
    import ctypes as C
    import torch
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    lib = _lib.load()
    ctx = pg.Context(0)
    w = wl.affine_pairs(n_pairs=300, seed=wl.SEED_BASE + 80)
    cm = pg.CostMatrix.of_transformations_and_gaps(ctx, w.subs, w.indel, w.gap_open)
    pk = pg.pack_pairs(w.pairs)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb), t(pk.out_off)]
    d_int = [torch.zeros(pk.npairs, dtype=torch.int32, device=dev) for _ in range(7)]
    d_out = [torch.zeros(pk.out_bytes, dtype=torch.uint8, device=dev) for _ in range(4)]
    P = lambda x: C.c_void_p(x.data_ptr())
    g = C.c_void_p()
    _lib.check(lib.poyalgn_batch_graph_create(
        ctx.handle, cm.handle, pk.npairs, pk.max_pair_len, pk.out_bytes, *(P(x) for x in d_in),
        *(P(x) for x in d_int[:6]), *(P(x) for x in d_out), P(d_int[6]), C.byref(g)))
    stream = torch.cuda.current_stream(0)
    rng = np.random.default_rng(81)
    for rnd in range(2):
        seqs = pk.seqs.copy()
        if rnd:  # new bases, same lengths and leading gaps
            pos = np.flatnonzero(seqs != 16)
            seqs[pos] = np.array([1, 2, 4, 8], np.uint8)[rng.integers(0, 4, len(pos))]
        d_in[0].copy_(torch.from_numpy(seqs))
        for x in d_out:
            x.zero_()
        _lib.check(lib.poyalgn_batch_graph_launch(g, C.c_void_p(stream.cuda_stream)))
        torch.cuda.synchronize()
        pairs = [(seqs[o:o + la], seqs[ob:ob + lb]) for o, la, ob, lb in
                 zip(pk.offa, pk.lena, pk.offb, pk.lenb)]
        ref = pg.median_batch(ctx, cm, pairs)
        assert np.array_equal(d_int[5].cpu().numpy(), ref.status)
        assert np.array_equal(d_int[0].cpu().numpy(), ref.cost)
        med = d_out[2].cpu().numpy()
        for k in range(pk.npairs):
            end = int(pk.out_off[k] + pk.cap[k])
            ml = int(ref.mlen[k])
            assert np.array_equal(med[end - ml:end], ref.pair(k).median), (rnd, k)
    lib.poyalgn_batch_graph_free(g)
    ctx.close()
