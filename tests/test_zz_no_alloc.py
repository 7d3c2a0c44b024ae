"""poyalgn_median_batch_device_noalloc against poyalgn_median_batch_device.

The no-allocation entry point keeps its scratch in static device memory; its
results must equal those of the context-based entry point, call after call.
This file sorts last so that it also runs after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

from cases import AFF_TCM, STD_TCM, edge_pairs, random_pairs

pytestmark = pytest.mark.gpu

OUT_NAMES = ("cost", "maxcost", "alen", "mlen", "wlen", "status", "passes")


def _batch(pairs):
    import torch
    import poy5_gb300 as pg
    pk = pg.pack_pairs(pairs)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb), t(pk.out_off)]
    return pk, d_in


def _outputs(pk, fill):
    import torch
    dev = torch.device("cuda", 0)
    ints = [torch.full((pk.npairs,), fill, dtype=torch.int32, device=dev) for _ in range(7)]
    byts = [torch.full((pk.out_bytes,), fill & 0xFF, dtype=torch.uint8, device=dev)
            for _ in range(4)]
    return ints, byts


def _run(fn, lead, pk, d_in, ints, byts):
    import torch
    from poy5_gb300 import _lib
    P = lambda x: C.c_void_p(x.data_ptr())
    stream = torch.cuda.current_stream(0)
    rc = fn(*lead, pk.npairs, pk.max_pair_len, pk.out_bytes, *(P(x) for x in d_in),
            *(P(x) for x in ints[:6]), *(P(x) for x in byts), P(ints[6]),
            C.c_void_p(stream.cuda_stream))
    _lib.check(rc)
    torch.cuda.synchronize(0)
    return [x.cpu().numpy() for x in ints], [x.cpu().numpy() for x in byts]


def _pair_views(pk, ints, byts):
    """Per pair, the bytes each output buffer holds (the right-aligned tail)."""
    alen, mlen, wlen = ints[2], ints[3], ints[4]
    out = []
    for k in range(pk.npairs):
        end = int(pk.out_off[k] + pk.lena[k] + pk.lenb[k] + 2)
        out.append((byts[0][end - alen[k]:end].tobytes(), byts[1][end - alen[k]:end].tobytes(),
                    byts[2][end - mlen[k]:end].tobytes(), byts[3][end - wlen[k]:end].tobytes()))
    return out


@pytest.mark.parametrize("affine", [False, True])
def test_noalloc_matches_context_entry_point(ctx, affine):
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    lib = _lib.load()
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    rng = np.random.default_rng(4242 + affine)
    batches = [edge_pairs() + random_pairs(rng, 300, maxlen=900),
               random_pairs(rng, 500, maxlen=1800)]
    for pairs in batches:  # two calls in a row, different batches
        pk, d_in = _batch(pairs)
        assert pk.max_pair_len <= 4096 and pk.npairs <= 16384
        want_i, want_b = _run(lib.poyalgn_median_batch_device, (ctx.handle, cm.handle),
                              pk, d_in, *_outputs(pk, 0))
        # outputs start as garbage: nothing the caller passes needs clearing
        got_i, got_b = _run(lib.poyalgn_median_batch_device_noalloc, (cm.handle,),
                            pk, d_in, *_outputs(pk, -77))
        assert np.array_equal(want_i[5], got_i[5]), "status"
        ok = want_i[5] == 0
        for name, w, g in zip(OUT_NAMES, want_i, got_i):
            assert np.array_equal(w[ok], g[ok]), name
        assert ok.sum() > 0.9 * pk.npairs
        views_w, views_g = _pair_views(pk, want_i, want_b), _pair_views(pk, got_i, got_b)
        for k in np.flatnonzero(ok):
            assert views_w[k] == views_g[k], k


def test_noalloc_rejects_oversized_batches(ctx):
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    lib = _lib.load()
    cm = pg.CostMatrix.of_list(ctx, STD_TCM, 0)
    null = C.c_void_p(0)
    good = C.c_void_p(1)  # never dereferenced: the size checks come first
    shapes = [(16385, 100, 1000, "POYALGN_NOALLOC_MAX_PAIRS"),
              (10, 4097, 1000, "POYALGN_NOALLOC_MAX_PAIR_LEN"),
              (10, 100, (4 << 20) + 1, "POYALGN_NOALLOC_MAX_OUT_BYTES")]
    for npairs, mpl, ob, limit in shapes:
        rc = lib.poyalgn_median_batch_device_noalloc(cm.handle, npairs, mpl, ob,
                                                     *([good] * 16), null, null)
        assert rc == -1
        assert limit in lib.poyalgn_last_error().decode()
