"""ctypes bindings to the oracle libraries (test infrastructure only).

``Oracle("port")`` loads ``oracle/libpoyoracle.so`` (the C restatement, built
from the repository's own sources on any machine); ``Oracle("ref")`` /
``Oracle("ref_long")`` load the
reference POY ``algn.c`` unit compiled in ``oracle/_ref`` (present only where
the POY sources were available). Both expose the same calls.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_PATHS = {
    "port": os.path.join(ORACLE_DIR, "libpoyoracle.so"),
    "ref": os.path.join(ORACLE_DIR, "_ref", "libpoyref.so"),
    "ref_long": os.path.join(ORACLE_DIR, "_ref", "libpoyref_long.so"),
}
_P = C.c_void_p
_I = C.c_int
_IP = C.POINTER(C.c_int)


def available(kind: str) -> bool:
    return os.path.exists(_PATHS[kind])


def build_port():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "build_oracle", os.path.join(ORACLE_DIR, "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build_port()


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


@dataclass
class Median:
    cost: int
    ea: np.ndarray      # aligned first input (caller order)
    eb: np.ndarray      # aligned second input
    median: np.ndarray  # ancestor (linear) / backtrace median (affine)
    medianwg: np.ndarray
    maxcost: int


class OracleError(RuntimeError):
    pass


class Oracle:
    def __init__(self, kind: str = "port"):
        if kind == "port" and not available("port"):
            build_port()
        path = _PATHS[kind]
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.kind = kind
        self.lib = C.CDLL(path)
        p = "orc_" if kind == "port" else "ref_"
        self._p = p
        L = self.lib
        getattr(L, p + "cm_new").restype = _P
        getattr(L, p + "cm_new").argtypes = [_P, _I, _I]
        getattr(L, p + "ws_new").restype = _P
        getattr(L, p + "last_error").restype = C.c_char_p
        self._ws = _P(getattr(L, p + "ws_new")())
        self._cms = {}

    def _f(self, name):
        return getattr(self.lib, self._p + name)

    def error(self) -> str:
        return self._f("last_error")().decode(errors="replace")

    def cm(self, tcm=None, alph=5, gap_open=0, subs=1, indel=2):
        """Cost matrix from a full alph x alph tcm (gap last) or subs/indel."""
        if tcm is None:
            tcm = [[0 if r == c else (indel if (r == alph - 1 or c == alph - 1)
                                      else subs) for c in range(alph)]
                   for r in range(alph)]
        flat = np.ascontiguousarray(np.asarray(tcm, dtype=np.int32).reshape(-1))
        key = (flat.tobytes(), alph, gap_open)
        if key not in self._cms:
            h = self._f("cm_new")(_ptr(flat), alph, gap_open)
            if not h:
                raise OracleError("cost matrix rejected")
            self._cms[key] = _P(h)
        return self._cms[key]

    def tables(self, cm):
        n = 8192
        cost = np.zeros(n, np.int32)
        worst = np.zeros(n, np.int32)
        tail = np.zeros(n, np.int32)
        prep = np.zeros(n, np.int32)
        med = np.zeros(n, np.uint8)
        info = np.zeros(6, np.int32)
        k = self._f("cm_tables")(cm, _ptr(cost), _ptr(med), _ptr(worst),
                                 _ptr(tail), _ptr(prep), _ptr(info))
        return dict(cost=cost[:k], median=med[:k], worst=worst[:k],
                    tail=tail[:k], prepend=prep[:k], lcm=int(info[0]),
                    gap=int(info[1]), a_sz=int(info[2]),
                    combinations=int(info[3]), cost_model=int(info[4]),
                    gap_open=int(info[5]))

    def median(self, cm, a, b, affine: bool) -> Median:
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        cap = len(a) + len(b) + 2
        ea, eb, med, mwg = (np.zeros(cap, np.uint8) for _ in range(4))
        cost, elen, mlen, wlen, mx = (_I() for _ in range(5))
        if affine:
            rc = self._f("median_affine")(
                cm, self._ws, _ptr(a), len(a), _ptr(b), len(b), C.byref(cost),
                _ptr(med), C.byref(mlen), _ptr(ea), _ptr(eb), C.byref(elen),
                _ptr(mwg), C.byref(wlen), C.byref(mx))
        else:
            rc = self._f("median_linear")(
                cm, self._ws, _ptr(a), len(a), _ptr(b), len(b), C.byref(cost),
                _ptr(ea), _ptr(eb), C.byref(elen), _ptr(med), C.byref(mlen),
                _ptr(mwg), C.byref(wlen), C.byref(mx))
        if rc:
            raise OracleError(self.error())
        n = elen.value
        return Median(cost.value, ea[:n].copy(), eb[:n].copy(),
                      med[:mlen.value].copy(), mwg[:wlen.value].copy(), mx.value)

    def cost_linear(self, cm, a, b, deltaw: int = -1) -> int:
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        c = _I()
        if self._f("cost_linear")(cm, self._ws, _ptr(a), len(a), _ptr(b),
                                  len(b), deltaw, C.byref(c)):
            raise OracleError(self.error())
        return c.value

    def cost_affine(self, cm, a, b) -> int:
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        c = _I()
        if self._f("cost_affine")(cm, self._ws, _ptr(a), len(a), _ptr(b),
                                  len(b), C.byref(c)):
            raise OracleError(self.error())
        return c.value

    def simple_2(self, cm, s1, s2, deltawh: int) -> int:
        s1 = np.ascontiguousarray(s1, np.uint8)
        s2 = np.ascontiguousarray(s2, np.uint8)
        c = _I()
        if self._f("simple_2")(cm, self._ws, _ptr(s1), len(s1), _ptr(s2),
                               len(s2), deltawh, C.byref(c)):
            raise OracleError(self.error())
        return c.value

    def backtrace_2d(self, cm, s1, s2, swap: int):
        s1 = np.ascontiguousarray(s1, np.uint8)
        s2 = np.ascontiguousarray(s2, np.uint8)
        cap = len(s1) + len(s2)
        r1 = np.zeros(cap, np.uint8)
        r2 = np.zeros(cap, np.uint8)
        n = _I()
        if self._f("backtrace_2d")(cm, self._ws, _ptr(s1), len(s1), _ptr(s2),
                                   len(s2), swap, _ptr(r1), _ptr(r2), cap,
                                   C.byref(n)):
            raise OracleError(self.error())
        return r1[:n.value].copy(), r2[:n.value].copy()

    def newkk_median(self, cm, a, b) -> Median:
        """DOS.median with use_ukk under an affine model (Algn_Newkk)."""
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        cap = len(a) + len(b) + 2
        ea, eb, anc, mwg = (np.zeros(cap, np.uint8) for _ in range(4))
        cost, elen, alen, wlen, mx = (_I() for _ in range(5))
        rc = self._f("newkk_median")(
            cm, _ptr(a), len(a), _ptr(b), len(b), C.byref(cost), _ptr(ea),
            _ptr(eb), C.byref(elen), _ptr(anc), C.byref(alen), _ptr(mwg),
            C.byref(wlen), C.byref(mx))
        if rc:
            raise OracleError(self.error())
        n = elen.value
        return Median(cost.value, ea[:n].copy(), eb[:n].copy(),
                      anc[:alen.value].copy(), mwg[:wlen.value].copy(), mx.value)

    # ---- port-only helpers ------------------------------------------------
    def set_check(self, on: bool):
        self.lib.orc_set_check(int(on))

    def schedule(self, cm, a, b, affine: bool):
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        it = _I()
        cells = C.c_int64()
        self.lib.orc_schedule(cm, int(affine), _ptr(a), len(a), _ptr(b),
                              len(b), C.byref(it), C.byref(cells))
        return it.value, cells.value

    def newkk_align(self, cm, s1, s2, swaped: int):
        """newkkonen_CAML_algn_affine + _backtrace_affine on (s1 shorter, s2):
        (cost, r1, r2, band passes, cells filled)."""
        s1 = np.ascontiguousarray(s1, np.uint8)
        s2 = np.ascontiguousarray(s2, np.uint8)
        cap = len(s1) + len(s2)
        r1 = np.zeros(cap, np.uint8)
        r2 = np.zeros(cap, np.uint8)
        cost, n, it = _I(), _I(), _I()
        cells = C.c_int64()
        if self.lib.orc_newkk_align(cm, _ptr(s1), len(s1), _ptr(s2), len(s2),
                                    swaped, C.byref(cost), _ptr(r1), _ptr(r2),
                                    C.byref(n), C.byref(it), C.byref(cells)):
            raise OracleError(self.error())
        return (cost.value, r1[:n.value].copy(), r2[:n.value].copy(), it.value,
                cells.value)

    def powell_3d(self, a, b, c, mm: int, go: int, ge: int):
        """powell_3D_align on three POY sequences (leading gap included):
        (cost, aligned a, aligned b, aligned c), each front to back with the
        leading gap. The reference build keeps its state in globals, so its
        calls must not overlap."""
        a, b, c = (np.ascontiguousarray(x, np.uint8) for x in (a, b, c))
        cap = len(a) + len(b) + len(c)
        ra, rb, rc = (np.zeros(cap, np.uint8) for _ in range(3))
        n, cost = _I(), _I()
        r = self._f("powell_3d")(_ptr(a), len(a), _ptr(b), len(b), _ptr(c), len(c),
                                 mm, go, ge, _ptr(ra), _ptr(rb), _ptr(rc),
                                 C.byref(n), C.byref(cost))
        if r:
            raise OracleError(self.error() if self.kind != "port" else f"powell_3d: {r}")
        k = n.value
        return cost.value, ra[:k].copy(), rb[:k].copy(), rc[:k].copy()

    def powell_3d_batch(self, seqs, off, lens, out_off, mm, go, ge, nthreads: int = 0):
        """orc_powell_3d_batch (the port only): arrays laid out as
        poyalgn_powell_3d_batch takes them; returns dict of cost, rlen,
        status, ra, rb, rc."""
        n = len(out_off)
        cap = np.asarray(lens, np.int64).reshape(-1, 3).sum(axis=1) if n else np.zeros(0)
        tot = int((np.asarray(out_off) + cap).max()) if n else 1
        ra, rb, rc = (np.zeros(tot, np.uint8) for _ in range(3))
        rlen, cost, status = (np.zeros(max(n, 1), np.int32) for _ in range(3))
        seqs, off, lens, out_off = (np.ascontiguousarray(a, dt) for a, dt in
                                    ((seqs, np.uint8), (off, np.int64), (lens, np.int32),
                                     (out_off, np.int64)))
        self.lib.orc_powell_3d_batch(n, _ptr(seqs), _ptr(off), _ptr(lens), mm, go, ge,
                                     _ptr(out_off), _ptr(ra), _ptr(rb), _ptr(rc), _ptr(rlen),
                                     _ptr(cost), _ptr(status), nthreads or (os.cpu_count() or 1))
        return dict(cost=cost[:n], rlen=rlen[:n], status=status[:n], ra=ra, rb=rb, rc=rc)

    def median_batch(self, cm, seqs_a, seqs_b, affine: bool, nthreads: int = 0):
        """DOS.median over many pairs on the host cores (OpenMP)."""
        la = np.array([len(s) for s in seqs_a], np.int32)
        lb = np.array([len(s) for s in seqs_b], np.int32)
        n = len(la)
        flat = np.concatenate([np.concatenate([a, b]) for a, b in
                               zip(seqs_a, seqs_b)]).astype(np.uint8)
        pair_len = (la + lb).astype(np.int64)
        offa = np.zeros(n, np.int64)
        offa[1:] = np.cumsum(pair_len)[:-1]
        offb = offa + la
        cap = (la + lb + 2).astype(np.int64)
        out_off = np.zeros(n, np.int64)
        out_off[1:] = np.cumsum(cap)[:-1]
        tot = int(cap.sum())
        ints = [np.zeros(n, np.int32) for _ in range(6)]
        bufs = [np.zeros(tot, np.uint8) for _ in range(4)]
        self.lib.orc_median_batch(
            cm, int(affine), n, _ptr(flat), _ptr(offa), _ptr(la), _ptr(offb),
            _ptr(lb), _ptr(out_off), *(_ptr(x) for x in ints[:5]),
            *(_ptr(x) for x in bufs), _ptr(ints[5]), nthreads)
        return dict(cost=ints[0], maxcost=ints[1], alen=ints[2], mlen=ints[3],
                    wlen=ints[4], status=ints[5], ea=bufs[0], eb=bufs[1],
                    med=bufs[2], mwg=bufs[3], out_off=out_off)


def compare_batch(ref: dict, ints, bufs, out_off, cap, chunk: int = 4096) -> dict:
    """Pairs of a GPU batch that differ from the oracle's median_batch on the
    same pairs. ints = (cost, maxcost, alen, mlen, wlen, status) and bufs =
    (ea, eb, med, mwg) as the batched entry points return them (each output
    ending at out_off + cap - 1); the oracle writes each from out_off on.
    Returns the count of differing pairs and the first few indices."""
    out_off = np.asarray(out_off, np.int64)
    cap = np.asarray(cap, np.int64)
    names = ("cost", "maxcost", "alen", "mlen", "wlen")
    bad = np.asarray(ref["status"]) != 0
    bad |= np.asarray(ints[5]) != 0
    for name, g in zip(names, ints[:5]):
        bad |= np.asarray(ref[name]) != np.asarray(g)
    lens = {"ea": ref["alen"], "eb": ref["alen"], "med": ref["mlen"], "mwg": ref["wlen"]}
    for lo in range(0, len(cap), chunk):
        hi = min(lo + chunk, len(cap))
        ok = ~bad[lo:hi]
        ks = np.arange(lo, hi)[ok]
        if len(ks) == 0:
            continue
        for name, g in zip(("ea", "eb", "med", "mwg"), bufs):
            n = np.asarray(lens[name])[ks].astype(np.int64)
            if n.sum() == 0:
                continue
            pair = np.repeat(np.arange(len(ks)), n)
            start = np.repeat(np.cumsum(n) - n, n)
            pos = np.arange(int(n.sum())) - start
            o = out_off[ks][pair] + pos
            gi = (out_off[ks] + cap[ks] - n)[pair] + pos
            diff = np.asarray(ref[name])[o] != np.asarray(g)[gi]
            if diff.any():
                bad[ks[np.unique(pair[diff])]] = True
    idx = np.flatnonzero(bad)
    return {"pairs": int(len(cap)), "mismatches": int(len(idx)),
            "first": [int(i) for i in idx[:8]]}
