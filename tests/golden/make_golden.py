"""Generate the golden fixtures from the reference POY algn.c build.

Run here, where the POY sources exist (``python oracle/build_oracle.py`` first
builds ``oracle/_ref/libpoyref.so``):

    python tests/golden/make_golden.py [--only newkk]

Each fixture holds the inputs of a set of pairs and what the reference's
SeqCS.DOS.median sequence of C calls returned for them (cost, aligned pair,
median, median with gaps, worst cost), plus the reference's cost tables.
``golden_newkk`` holds DOS.median with use_ukk (affine): the pair aligned by
src/newkkonen.c, then ancestor_2 / median_2_with_gaps / max_cost_2.
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


def main():
    ref = Oracle("ref")
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "newkk":
        make_newkk(ref)
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


if __name__ == "__main__":
    main()
