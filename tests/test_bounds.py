"""Device-side bounds of the device-pointer batch entry points.

poyalgn_median_batch_device, poyalgn_median_batch_device_noalloc and
poyalgn_distance_batch_device take the caller's word for the batch shape
(max_pair_len, out_bytes), which sizes the direction slabs, the output slots
and the affine row-0 shadow. A pair outside that shape must fail with its own
status and leave every buffer alone, while the other pairs of the batch give
their normal results. The buffers here are allocated at the true size, so a
missing check would show as overwritten bytes, never as a fault.
"""
import ctypes as C

import numpy as np
import pytest

from cases import AFF_TCM, STD_TCM, random_pairs

pytestmark = pytest.mark.gpu

FILL = 0x5A


def _dev(pk):
    import torch
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb), t(pk.out_off)]
    ints = [torch.full((pk.npairs,), -77, dtype=torch.int32, device=dev) for _ in range(7)]
    byts = [torch.full((pk.out_bytes,), FILL, dtype=torch.uint8, device=dev) for _ in range(4)]
    return d_in, ints, byts


def _call(fn, lead, pk, max_pair_len, out_bytes):
    import torch
    from poy5_gb300 import _lib
    d_in, ints, byts = _dev(pk)
    P = lambda x: C.c_void_p(x.data_ptr())
    rc = fn(*lead, pk.npairs, max_pair_len, out_bytes, *(P(x) for x in d_in),
            *(P(x) for x in ints[:6]), *(P(x) for x in byts), P(ints[6]),
            C.c_void_p(torch.cuda.current_stream(0).cuda_stream))
    _lib.check(rc)
    torch.cuda.synchronize(0)
    return [x.cpu().numpy() for x in ints], [x.cpu().numpy() for x in byts]


def _shape(pairs):
    """The batch with its longest pair moved to the front and the declared
    shape cut so that pair 0 is one position too long and the last pair's
    output slot ends one byte past out_bytes."""
    import poy5_gb300 as pg
    lens = [len(a) + len(b) for a, b in pairs]
    k = int(np.argmax(lens))
    pairs = [pairs[k]] + pairs[:k] + pairs[k + 1:]
    pk = pg.pack_pairs(pairs)
    plen = pk.lena.astype(np.int64) + pk.lenb
    second = int(np.sort(plen)[-2])
    assert plen[0] > second, "need a unique longest pair"
    return pk, int(plen[0]) - 1, int(pk.out_bytes) - 1


@pytest.mark.parametrize("affine", [False, True])
@pytest.mark.parametrize("entry", ["device", "noalloc"])
def test_pairs_outside_declared_shape_fail_alone(ctx, affine, entry):
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    lib = _lib.load()
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    cm = pg.CostMatrix.of_list(ctx, tcm, go)
    rng = np.random.default_rng(777 + affine)
    pairs = random_pairs(rng, 200, maxlen=700)
    pairs[0] = (pairs[0][0], np.concatenate([pairs[0][1], pairs[0][1][1:]]).astype(np.uint8))
    pk, short_len, short_out = _shape(pairs)
    want_i, want_b = _call(lib.poyalgn_median_batch_device, (ctx.handle, cm.handle), pk,
                           pk.max_pair_len, pk.out_bytes)
    fn, lead = ((lib.poyalgn_median_batch_device, (ctx.handle, cm.handle)) if entry == "device"
                else (lib.poyalgn_median_batch_device_noalloc, (cm.handle,)))
    got_i, got_b = _call(fn, lead, pk, short_len, short_out)
    last = pk.npairs - 1
    assert got_i[5][0] == -6, got_i[5][0]          # POYALGN_PAIR_TOO_LONG
    assert got_i[5][last] == -2, got_i[5][last]     # POYALGN_PAIR_CAPACITY
    for k in (0, last):                             # their slots are untouched
        lo, hi = int(pk.out_off[k]), int(pk.out_off[k] + pk.cap[k])
        for buf in got_b:
            assert np.all(buf[lo:min(hi, len(buf))] == FILL), k
    rest = np.ones(pk.npairs, bool)
    rest[[0, last]] = False
    assert np.array_equal(want_i[5][rest], got_i[5][rest])
    ok = rest & (want_i[5] == 0)
    assert ok.sum() > 0.9 * rest.sum()
    for w, g in zip(want_i[:5], got_i[:5]):
        assert np.array_equal(w[ok], g[ok])
    for k in np.flatnonzero(ok):
        lo, hi = int(pk.out_off[k]), int(pk.out_off[k] + pk.cap[k])
        for w, g in zip(want_b, got_b):
            assert np.array_equal(w[lo:hi], g[lo:hi]), k


def test_distance_pair_longer_than_declared_fails_alone(ctx):
    import torch
    import poy5_gb300 as pg
    from poy5_gb300 import _lib
    lib = _lib.load()
    cm = pg.CostMatrix.of_list(ctx, STD_TCM, 0)
    rng = np.random.default_rng(91)
    pairs = random_pairs(rng, 100, maxlen=600)
    pairs[0] = (pairs[0][0], np.concatenate([pairs[0][1], pairs[0][1][1:]]).astype(np.uint8))
    pk, short_len, _ = _shape(pairs)
    want_cost, want_status = pg.distance_batch(ctx, cm, pk)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_in = [t(pk.seqs), t(pk.offa), t(pk.lena), t(pk.offb), t(pk.lenb)]
    cost = torch.full((pk.npairs,), -77, dtype=torch.int32, device=dev)
    status = torch.full((pk.npairs,), -77, dtype=torch.int32, device=dev)
    P = lambda x: C.c_void_p(x.data_ptr())
    _lib.check(lib.poyalgn_distance_batch_device(
        ctx.handle, cm.handle, pk.npairs, short_len, *(P(x) for x in d_in), 0, P(cost),
        P(status), C.c_void_p(torch.cuda.current_stream(0).cuda_stream)))
    torch.cuda.synchronize(0)
    cost, status = cost.cpu().numpy(), status.cpu().numpy()
    assert status[0] == -6
    assert np.array_equal(status[1:], want_status[1:])
    assert np.array_equal(cost[1:], want_cost[1:])
