"""The kernels' lane-pipeline algorithm, replayed on the host (no GPU).

libpa_emul.so compiles the same step and traceback functions the CUDA
kernels run (poy5_gb300/csrc/pa_core.cuh) plus the library's own cost-table
builder, and replays P pipeline lanes one at a time. These tests pin that
algorithm to the reference (golden fixtures) and to the oracle, so a GPU run
only has to confirm the CUDA mechanics.
"""
import ctypes as C

import numpy as np
import pytest

import golden_lib
from cases import AFF_TCM, STD_TCM, edge_pairs, random_pairs
from conftest import build_emulator

_P = C.c_void_p


@pytest.fixture(scope="module")
def emul():
    lib = C.CDLL(build_emulator())
    lib.pa_emul_new.restype = _P
    lib.pa_emul_new.argtypes = [_P, C.c_int, C.c_int]
    lib.pa_emul_free.argtypes = [_P]
    lib.pa_emul_set_row_tile.argtypes = [_P, C.c_int]
    return lib


def _ptr(a):
    return a.ctypes.data_as(_P)


class Emu:
    def __init__(self, lib, tcm, go, row_tile=1):
        self.lib = lib
        flat = np.ascontiguousarray(np.asarray(tcm, np.int32).reshape(-1))
        self.h = _P(lib.pa_emul_new(_ptr(flat), int(np.asarray(tcm).shape[0]), go))
        assert self.h
        lib.pa_emul_set_row_tile(self.h, row_tile)
        self.affine = go > 0

    def tables(self):
        n = 8192
        cost, worst, tail, prep = (np.zeros(n, np.int32) for _ in range(4))
        med = np.zeros(n, np.uint8)
        info = np.zeros(6, np.int32)
        k = self.lib.pa_emul_tables(self.h, _ptr(cost), _ptr(med), _ptr(worst), _ptr(tail),
                                    _ptr(prep), _ptr(info))
        return dict(cost=cost[:k], median=med[:k], worst=worst[:k], tail=tail[:k],
                    prepend=prep[:k])

    def median(self, a, b):
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        cap = len(a) + len(b) + 2
        bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
        res = np.zeros(4, np.int32)
        cost, ps, lc = C.c_int(), C.c_int(), C.c_int()
        rc = self.lib.pa_emul_median(self.h, int(self.affine), _ptr(a), len(a), _ptr(b), len(b),
                                     C.byref(cost), *(_ptr(x) for x in bufs), cap, _ptr(res),
                                     C.byref(ps), C.byref(lc))
        assert rc == 0, rc
        al, ml, wl, mx = (int(x) for x in res)
        return (cost.value, bufs[0][cap - al:], bufs[1][cap - al:], bufs[2][cap - ml:],
                bufs[3][cap - wl:], mx, lc.value)

    def __del__(self):
        self.lib.pa_emul_free(self.h)


@pytest.mark.parametrize("name", golden_lib.NAMES)
def test_pipeline_matches_golden(emul, name):
    g = golden_lib.load(name)
    e = Emu(emul, g.tcm, g.gap_open)
    t = e.tables()
    for key, want in g.tables.items():
        assert np.array_equal(t[key], want), key
    for k, (a, b) in enumerate(g.pairs):
        cost, ea, eb, med, mwg, mx, _ = e.median(a, b)
        bad = golden_lib.mismatches(g, k, cost, ea, eb, med, mwg, mx)
        assert not bad, (name, k, bad)


@pytest.mark.parametrize("affine,row_tile", [(False, 1), (True, 1), (True, 0)])
def test_pipeline_matches_oracle_random(emul, oracle, affine, row_tile):
    """row_tile 0 keeps lean (gap-free) affine pairs on the lane pipeline,
    whose ladder interleaves R = 3 shapes with the R = 2 and 4 ones."""
    rng = np.random.default_rng(314 + affine)
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    e = Emu(emul, tcm, go, row_tile)
    cm = oracle.cm(tcm=tcm, gap_open=go)
    classes = set()
    for a, b in edge_pairs() + random_pairs(rng, 300, maxlen=700):
        cost, ea, eb, med, mwg, mx, cls = e.median(a, b)
        r = oracle.median(cm, a, b, affine)
        classes.add(cls)
        assert (cost, mx) == (r.cost, r.maxcost)
        assert np.array_equal(ea, r.ea) and np.array_equal(eb, r.eb)
        assert np.array_equal(med, r.median) and np.array_equal(mwg, r.medianwg)
    assert len(classes) >= 4  # single-warp and multi-warp pipelines exercised


def test_pipeline_random_tables(emul, oracle):
    rng = np.random.default_rng(8)
    for t in range(12):
        M = rng.integers(1, 5, (5, 5))
        M = np.triu(M) + np.triu(M, 1).T
        if t % 2:
            np.fill_diagonal(M, 0)
        go = 2 if t % 3 == 0 else 0
        e = Emu(emul, M, go)
        cm = oracle.cm(tcm=M.tolist(), gap_open=go)
        for a, b in random_pairs(rng, 10, maxlen=200):
            cost, ea, eb, med, mwg, mx, _ = e.median(a, b)
            r = oracle.median(cm, a, b, go > 0)
            assert (cost, mx) == (r.cost, r.maxcost)
            assert np.array_equal(med, r.median) and np.array_equal(ea, r.ea)


def test_pair_bounds_status(emul):
    """prep_kernel's per-pair guard (pair_bounds_status): a pair longer than
    the batch's declared max_pair_len (-6) or whose output slot runs past
    out_bytes (-2) fails before it touches a slab, an output or the shadow."""
    f = emul.pa_emul_pair_bounds
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_int]
    cases = [
        ((100, 200, 300, 0, 302, 1), 0),        # exactly fits both bounds
        ((100, 201, 300, 0, 10_000, 1), -6),    # one position past max_pair_len
        ((100, 200, 300, 0, 301, 1), -2),       # slot one byte past out_bytes
        ((100, 200, 300, 500, 801, 1), -2),
        ((100, 200, 300, 499, 801, 1), 0),
        ((100, 200, 300, -1, 10_000, 1), -2),   # negative offset
        ((100, 200, 300, 1 << 40, 0, 0), 0),    # no outputs: out_off unused
        ((-1, 5, 300, 0, 100, 1), -6),          # negative length
        ((2_000_000_000, 2_000_000_000, 2_147_483_647, 0, 1 << 40, 1), -6),  # no int overflow
    ]
    for args, want in cases:
        assert f(*args) == want, (args, want)


def test_window_traceback_on_wide_classes(emul, oracle):
    """Longer, more divergent linear pairs, whose final bands need pipelines
    of 64-256 lanes: their tracebacks run through the shared-memory window
    (LinDmWindow, refilled every LW_DIAG anti-diagonals) and must match the
    oracle byte for byte."""
    from poy5_gb300 import workloads as wl
    rng = np.random.default_rng(77)
    e = Emu(emul, STD_TCM, 0)
    cm = oracle.cm(tcm=STD_TCM)
    classes = set()
    for L, sub, ind in ((1500, 0.15, 0.03), (2500, 0.2, 0.05), (3000, 0.1, 0.08)):
        core = wl.random_bases(rng, L)
        a = wl.with_gap(core)
        b = wl.with_gap(wl.mutate(rng, core, sub, ind))
        cost, ea, eb, med, mwg, mx, cls = e.median(a, b)
        classes.add(cls)
        r = oracle.median(cm, a, b, False)
        assert (cost, mx) == (r.cost, r.maxcost)
        assert np.array_equal(ea, r.ea) and np.array_equal(eb, r.eb)
        assert np.array_equal(med, r.median) and np.array_equal(mwg, r.medianwg)
    assert max(classes) >= 6, classes


def test_window_traceback_on_every_class(emul, oracle):
    """The deferred linear traceback runs every class's walk through the
    shared-memory window, also for pipelines of fewer than 64 lane-rows,
    whose window holds whole anti-diagonals with rows aliased modulo P R:
    golden pairs and random pairs of every width against the references."""
    emul.pa_emul_set_window.argtypes = [_P, C.c_int]
    for name in ("golden_linear", "golden_plain_pairs"):
        g = golden_lib.load(name)
        e = Emu(emul, g.tcm, g.gap_open)
        emul.pa_emul_set_window(e.h, 1)
        for k, (a, b) in enumerate(g.pairs):
            cost, ea, eb, med, mwg, mx, _ = e.median(a, b)
            bad = golden_lib.mismatches(g, k, cost, ea, eb, med, mwg, mx)
            assert not bad, (name, k, bad)
    rng = np.random.default_rng(515)
    e = Emu(emul, STD_TCM, 0)
    emul.pa_emul_set_window(e.h, 1)
    cm = oracle.cm(tcm=STD_TCM)
    classes = set()
    for a, b in edge_pairs() + random_pairs(rng, 300, maxlen=700):
        cost, ea, eb, med, mwg, mx, cls = e.median(a, b)
        classes.add(cls)
        r = oracle.median(cm, a, b, False)
        assert (cost, mx) == (r.cost, r.maxcost)
        assert np.array_equal(ea, r.ea) and np.array_equal(eb, r.eb)
        assert np.array_equal(med, r.median) and np.array_equal(mwg, r.medianwg)
    assert min(classes) == 0 and len(classes) >= 5, classes


@pytest.mark.parametrize("row_tile", [0, 1])
def test_window_traceback_lean_affine(emul, oracle, row_tile):
    """Lean affine tracebacks (gap-free pairs on the lane pipeline, one byte
    per cell) through the same window as the deferred lean traceback runs
    them, on every affine class including the R = 3 ones, whose P R is not
    a power of two; row-tile fills through the window of whole rows the
    deferred row-tile traceback uses (AffDmRowWindow)."""
    emul.pa_emul_set_window.argtypes = [_P, C.c_int]
    for name in ("golden_affine", "golden_affine_pairs"):
        g = golden_lib.load(name)
        e = Emu(emul, g.tcm, g.gap_open, row_tile)
        emul.pa_emul_set_window(e.h, 1)
        for k, (a, b) in enumerate(g.pairs):
            cost, ea, eb, med, mwg, mx, _ = e.median(a, b)
            bad = golden_lib.mismatches(g, k, cost, ea, eb, med, mwg, mx)
            assert not bad, (name, k, bad)
    rng = np.random.default_rng(616 + row_tile)
    e = Emu(emul, AFF_TCM, 3, row_tile)
    emul.pa_emul_set_window(e.h, 1)
    cm = oracle.cm(tcm=AFF_TCM, gap_open=3)
    classes = set()
    for a, b in random_pairs(rng, 300, maxlen=900, kinds=2):  # gap-free kinds: lean
        try:
            r = oracle.median(cm, a, b, True)
        except Exception:
            continue
        cost, ea, eb, med, mwg, mx, cls = e.median(a, b)
        classes.add(cls)
        assert (cost, mx) == (r.cost, r.maxcost)
        assert np.array_equal(ea, r.ea) and np.array_equal(eb, r.eb)
        assert np.array_equal(med, r.median) and np.array_equal(mwg, r.medianwg)
    if row_tile == 0:
        assert {1, 3, 5} & classes and len(classes) >= 5, classes  # R = 3 classes walked


def _pass_cases(rng):
    from cases import edge_pairs, mutate, rseq
    pairs = edge_pairs() + random_pairs(rng, 300, maxlen=700)
    for _ in range(120):  # unequal lengths, gapped states, tiny sequences
        la = int(rng.integers(1, 400))
        a = rseq(rng, la, amb=0.05, gapp=float(rng.choice([0.0, 0.1])))
        b = mutate(rng, a, 0.2, float(rng.choice([0.0, 0.05, 0.2])))
        if rng.random() < 0.3:
            b = np.concatenate([b, rseq(rng, int(rng.integers(1, 300)))[1:]])
        pairs.append((a, b) if rng.random() < 0.5 else (b, a))
    for name in ("golden_linear", "golden_affine", "golden_affine_pairs"):
        if name in golden_lib.NAMES:
            pairs += list(golden_lib.load(name).pairs)
    return pairs


@pytest.mark.parametrize("affine", [False, True])
def test_every_pass_reports_at_least_the_length_difference(emul, affine):
    """The bound the kernels use to skip the doubling's first passes
    (unstoppable_passes): every pass's gap count is at least n - m, so a
    pass with T below 3 (n - m) + 4 (linear) / + 2 (affine) cannot stop."""
    emul.pa_emul_set_skip.argtypes = [_P, C.c_int]
    f = emul.pa_emul_aff_passes if affine else emul.pa_emul_lin_passes
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    e = Emu(emul, tcm, go)
    emul.pa_emul_set_skip(e.h, 0)
    rng = np.random.default_rng(900 + affine)
    Ts, gaps, cls = (np.zeros(64, np.int32) for _ in range(3))
    checked = 0
    for a, b in _pass_cases(rng):
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        if affine:
            np_ = f(e.h, _ptr(a), len(a), _ptr(b), len(b), _ptr(Ts), _ptr(gaps), 64)
        else:
            np_ = f(e.h, _ptr(a), len(a), _ptr(b), len(b), _ptr(Ts), _ptr(gaps), _ptr(cls), 64)
        d = abs(len(a) - len(b))
        for j in range(max(np_, 0)):
            assert gaps[j] >= d, (len(a), len(b), j, int(Ts[j]), int(gaps[j]))
            checked += 1
    assert checked > 1000


@pytest.mark.parametrize("affine", [False, True])
def test_skipped_passes_change_nothing(emul, affine):
    """Starting after the unstoppable passes gives every output of the full
    doubling, and the same pass count."""
    emul.pa_emul_set_skip.argtypes = [_P, C.c_int]
    tcm, go = (AFF_TCM, 3) if affine else (STD_TCM, 0)
    full, skip = Emu(emul, tcm, go), Emu(emul, tcm, go)
    emul.pa_emul_set_skip(full.h, 0)
    emul.pa_emul_set_skip(skip.h, 1)
    rng = np.random.default_rng(910 + affine)
    skipped = 0
    for a, b in _pass_cases(rng):
        try:
            r0 = _median_passes(emul, full, a, b)
        except AssertionError:
            continue
        r1 = _median_passes(emul, skip, a, b)
        assert r0[0] == r1[0] and r0[2] == r1[2] and r0[-1] == r1[-1], (len(a), len(b))
        for x, y in zip(r0[1], r1[1]):
            assert np.array_equal(x, y), (len(a), len(b))
        skipped += 1
    assert skipped > 300


def _median_passes(lib, e, a, b):
    a = np.ascontiguousarray(a, np.uint8)
    b = np.ascontiguousarray(b, np.uint8)
    cap = len(a) + len(b) + 2
    bufs = [np.zeros(cap, np.uint8) for _ in range(4)]
    res = np.zeros(4, np.int32)
    cost, ps, lc = C.c_int(), C.c_int(), C.c_int()
    rc = lib.pa_emul_median(e.h, int(e.affine), _ptr(a), len(a), _ptr(b), len(b),
                            C.byref(cost), *(_ptr(x) for x in bufs), cap, _ptr(res),
                            C.byref(ps), C.byref(lc))
    assert rc == 0, rc
    return (cost.value, bufs, tuple(res), ps.value)


def test_host_skip_accounting_matches_kernels(emul):
    """schedule.unstoppable_passes (GCUPS accounting) is the kernels' rule."""
    from poy5_gb300 import schedule
    rng = np.random.default_rng(920)
    la = rng.integers(1, 5000, 4000)
    lb = np.where(rng.random(4000) < 0.5, la + rng.integers(-30, 30, 4000),
                  rng.integers(1, 5000, 4000)).clip(1, None)
    for affine in (False, True):
        for mnz in (1, 2, 3):
            got = schedule.unstoppable_passes(la, lb, mnz, affine)
            m, n = np.minimum(la, lb), np.maximum(la, lb)
            want = [emul.pa_emul_unstoppable(int((b - a + 1) * mnz), int(a), int(b), int(affine))
                    for a, b in zip(m, n)]
            assert np.array_equal(got, want), (affine, mnz)
            assert got.max() <= 2
