"""Generate the golden fixtures from the reference POY algn.c build.

Run here, where the POY sources exist (``python oracle/build_oracle.py`` first
builds ``oracle/_ref/libpoyref.so``):

    python tests/golden/make_golden.py [--only newkk|powell3d]

Each fixture holds the inputs of a set of pairs and what the reference's
SeqCS.DOS.median sequence of C calls returned for them (cost, aligned pair,
median, median with gaps, worst cost), plus the reference's cost tables.
``golden_newkk`` holds DOS.median with use_ukk (affine): the pair aligned by
src/newkkonen.c, then ancestor_2 / median_2_with_gaps / max_cost_2.
``golden_powell3d`` holds powell_3D_align (src/ukkCommon.c, src/ukk.checkp.c)
on triples: the cost and the three aligned sequences.
The GPU tests compare against these files directly, so parity is pinned to
the reference itself and not only to the C restatement.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from cases import AFF_TCM, STD_TCM, edge_pairs, random_pairs  # noqa: E402
from oracle_lib import Oracle  # noqa: E402


def pack(outs):
    lens = np.array([len(o) for o in outs], np.int64)
    off = np.zeros(len(outs) + 1, np.int64)
    off[1:] = np.cumsum(lens)
    return np.concatenate(outs).astype(np.uint8) if outs else np.zeros(0, np.uint8), off


def make(name, ref, tcm, gap_open, pairs, newkk=False):
    cm = ref.cm(tcm=tcm, gap_open=gap_open)
    if newkk:  # DOS.median with use_ukk (Algn_Newkk, src/newkkonen.c)
        res = [ref.newkk_median(cm, a, b) for a, b in pairs]
    else:
        res = [ref.median(cm, a, b, gap_open > 0) for a, b in pairs]
    a_flat, a_off = pack([a for a, _ in pairs])
    b_flat, b_off = pack([b for _, b in pairs])
    fields = {}
    for key in ("ea", "eb", "median", "medianwg"):
        fields[key], fields[key + "_off"] = pack([getattr(r, key) for r in res])
    t = ref.tables(cm)
    np.savez_compressed(
        os.path.join(HERE, f"{name}.npz"), tcm=np.asarray(tcm, np.int32),
        gap_open=gap_open, a=a_flat, a_off=a_off, b=b_flat, b_off=b_off,
        cost=np.array([r.cost for r in res], np.int32),
        maxcost=np.array([r.maxcost for r in res], np.int32),
        t_cost=t["cost"], t_median=t["median"], t_worst=t["worst"],
        t_tail=t["tail"], t_prepend=t["prepend"], **fields)
    print(name, len(pairs), "pairs")


def make_newkk(ref):
    rng = np.random.default_rng(4242)
    pairs = edge_pairs() + random_pairs(rng, 150, maxlen=400)
    from poy5_gb300 import workloads as wl
    pairs += wl.affine_pairs(n_pairs=16).pairs
    make("golden_newkk", ref, AFF_TCM, 3, pairs, newkk=True)


def powell_cases(rng, n_random=60):
    """Triples for the three-sequence alignment fixture: edge cases under
    three cost models, random triples of 0-80 positions at several
    divergences and cost models, and readjust-shaped triples."""
    G = 16
    edge = [([G], [G], [G]), ([G, 1], [G], [G]), ([G], [G, 1, 2], [G, 4]),
            ([G, 1, 2, 4], [G, 1, 2, 4], [G, 1, 2, 4]), ([G, 1, 2, 4], [G, 1, 2, 4], [G, 1, 2, 8]),
            ([G, 1], [G, 2], [G, 4]), ([G, 1, 1, 1, 1], [G, 2, 2, 2, 2], [G, 4, 4, 4, 4]),
            ([G, 3, 5, 15], [G, 1, 4, 8], [G, 2, 4, 8]), ([G, 1, 2, 4, 8], [G], [G, 1, 2, 4, 8])]
    cases = [(t, c) for t in edge for c in ((1, 0, 2), (1, 3, 1), (2, 1, 1))]

    def mut(s, div):
        out = []
        for x in s:
            r = rng.random()
            if r < div / 4:
                continue
            if r < div / 2:
                out.append(int(rng.choice([1, 2, 4, 8])))
            out.append(x if rng.random() > div else int(rng.choice([1, 2, 4, 8])))
        return out

    for _ in range(n_random):
        L = int(rng.integers(0, 80))
        div = float(rng.choice([0.02, 0.1, 0.3, 0.6]))
        base = rng.choice([1, 2, 4, 8], L).tolist()
        t = []
        for _ in range(3):
            s = [G] + mut(base, div)
            for i in range(1, len(s)):
                if rng.random() < 0.05:
                    s[i] |= int(rng.choice([1, 2, 4, 8, 16]))
            t.append(s)
        c = (int(rng.choice([1, 2, 3])), int(rng.choice([0, 0, 1, 2, 3])),
             int(rng.choice([1, 2, 3])))
        cases.append((tuple(t), c))
    from poy5_gb300 import workloads as wl
    w = wl.readjust_triples(n_triples=8)
    cases += [(t, (w.mm, w.go, w.ge)) for t in w.triples]
    return cases


def make_powell3d(ref):
    """golden_powell3d: powell_3D_align (src/ukkCommon.c:109) on triples,
    the cost and the three aligned sequences the reference returned."""
    rng = np.random.default_rng(31337)
    cases = powell_cases(rng)
    res = [ref.powell_3d(*t, *c) for t, c in cases]
    fields = {}
    for j, key in enumerate(("a", "b", "c")):
        fields[key], fields[key + "_off"] = pack([np.asarray(t[j], np.uint8) for t, _ in cases])
        fields["r" + key], fields["r" + key + "_off"] = pack([r[1 + j] for r in res])
    np.savez_compressed(os.path.join(HERE, "golden_powell3d.npz"),
                        costs=np.array([c for _, c in cases], np.int32),
                        cost=np.array([r[0] for r in res], np.int32), **fields)
    print("golden_powell3d", len(cases), "triples")


def main():
    ref = Oracle("ref")
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "newkk":
        make_newkk(ref)
        return
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "powell3d":
        make_powell3d(ref)
        return
    rng = np.random.default_rng(777)
    lin = edge_pairs() + random_pairs(rng, 120, maxlen=400)
    aff = edge_pairs() + random_pairs(rng, 120, maxlen=400)
    make("golden_linear", ref, STD_TCM, 0, lin)
    make("golden_affine", ref, AFF_TCM, 3, aff)
    # workload-shaped samples
    from poy5_gb300 import workloads as wl
    w1 = wl.plain_pairs(n_pairs=24)
    make("golden_plain_pairs", ref, STD_TCM, 0, w1.pairs)
    w2 = wl.affine_pairs(n_pairs=24)
    make("golden_affine_pairs", ref, AFF_TCM, 3, w2.pairs)
    make_newkk(ref)
    make_powell3d(ref)


if __name__ == "__main__":
    main()
