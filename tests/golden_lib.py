"""Loader for the golden fixtures generated by tests/golden/make_golden.py."""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["golden_linear", "golden_affine", "golden_plain_pairs", "golden_affine_pairs"]
# DOS.median with use_ukk (Algn_Newkk), affine
NEWKK_NAMES = ["golden_newkk"]


@dataclass
class Golden:
    name: str
    tcm: np.ndarray
    gap_open: int
    pairs: list
    cost: np.ndarray
    maxcost: np.ndarray
    ea: list
    eb: list
    median: list
    medianwg: list
    tables: dict

    @property
    def affine(self) -> bool:
        return self.gap_open > 0


def _unpack(flat, off):
    return [flat[off[i]:off[i + 1]] for i in range(len(off) - 1)]


def load(name: str) -> Golden:
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    a = _unpack(z["a"], z["a_off"])
    b = _unpack(z["b"], z["b_off"])
    return Golden(name, z["tcm"], int(z["gap_open"]), list(zip(a, b)), z["cost"],
                  z["maxcost"], _unpack(z["ea"], z["ea_off"]), _unpack(z["eb"], z["eb_off"]),
                  _unpack(z["median"], z["median_off"]),
                  _unpack(z["medianwg"], z["medianwg_off"]),
                  {k: z["t_" + k] for k in ("cost", "median", "worst", "tail", "prepend")})


def mismatches(g: Golden, k: int, cost, ea, eb, med, mwg, maxcost) -> list:
    bad = []
    if cost != g.cost[k]:
        bad.append("cost")
    if maxcost != g.maxcost[k]:
        bad.append("maxcost")
    for nm, got, want in (("ea", ea, g.ea[k]), ("eb", eb, g.eb[k]),
                          ("median", med, g.median[k]), ("medianwg", mwg, g.medianwg[k])):
        if not np.array_equal(np.asarray(got, np.uint8), want):
            bad.append(nm)
    return bad
