"""Seeded synthetic workloads (the reference ships no data for this path).

Sequences are POY bitset states with the leading gap. Seeds are
``SEED_BASE + k`` for workload k = 1..5:

1. ``plain_pairs``: 4,096 independent pairs, lengths U[200, 600], bases i.i.d.
   uniform over {A, C, G, T}, 1% of positions replaced by a uniform IUPAC
   ambiguity; linear costs (substitution 1, indel 2).
2. ``affine_pairs``: 65,536 pairs, first length round(lognormal(ln 800,
   0.8)) clipped to [50, 4000], second derived by 10% substitutions and indel
   events at rate 0.02 per site with geometric lengths (mean 3); affine costs
   (gap opening 3, extension 1, substitution 1).
3. ``yule_tree``: 256-taxon Yule tree, exponential branch lengths (mean
   0.05), uniform root of length 1,500, Jukes-Cantor substitutions, indels at
   0.2x the substitution rate (geometric lengths, mean 3); linear 1/2.
4. ``serving_requests``: Poisson arrivals, 1..64 pairs per request, lengths
   lognormal(ln 1000, 0.8) clipped to [100, 5000] at 30% divergence; affine.
5. ``long_pairs``: 512 pairs of 20-50 kb at 15% substitutions, 2% indels;
   linear 1/2.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEED_BASE = 20261203
GAP = 16
BASES = np.array([1, 2, 4, 8], np.uint8)
AMBIG = np.array([3, 5, 6, 7, 9, 10, 11, 12, 13, 14, 15], np.uint8)


def with_gap(s: np.ndarray) -> np.ndarray:
    out = np.empty(len(s) + 1, np.uint8)
    out[0] = GAP
    out[1:] = s
    return out


def random_bases(rng: np.random.Generator, n: int) -> np.ndarray:
    return BASES[rng.integers(0, 4, n)]


def substitute(rng: np.random.Generator, s: np.ndarray, rate: float) -> np.ndarray:
    """Replace a `rate` fraction of bases by a different base."""
    s = s.copy()
    hit = np.nonzero(rng.random(len(s)) < rate)[0]
    if len(hit):
        idx = np.log2(np.maximum(s[hit], 1)).astype(np.int64) & 3
        s[hit] = BASES[(idx + rng.integers(1, 4, len(hit))) & 3]
    return s


def indels(rng: np.random.Generator, s: np.ndarray, rate: float,
           mean_len: float = 3.0) -> np.ndarray:
    """Insert/delete runs at `rate` events per site, geometric lengths."""
    n = len(s)
    k = rng.binomial(n, rate) if n else 0
    if k == 0:
        return s
    pos = np.sort(rng.integers(0, n + 1, k))
    lens = rng.geometric(1.0 / mean_len, k)
    ins = rng.random(k) < 0.5
    parts = []
    cur = 0
    for p, ln, is_ins in zip(pos, lens, ins):
        if p < cur:
            p = cur
        parts.append(s[cur:p])
        if is_ins:
            parts.append(random_bases(rng, int(ln)))
            cur = p
        else:
            cur = min(n, p + int(ln))
    parts.append(s[cur:])
    return np.concatenate(parts) if parts else s


def mutate(rng, s, sub_rate, indel_rate, mean_len=3.0):
    return indels(rng, substitute(rng, s, sub_rate), indel_rate, mean_len)


@dataclass
class PairWorkload:
    name: str
    pairs: list          # [(a, b)] bitset sequences with leading gap
    subs: int
    indel: int
    gap_open: int        # 0 = linear

    @property
    def affine(self) -> bool:
        return self.gap_open > 0

    def cells_full(self) -> int:
        return int(sum((len(a) - 1) * (len(b) - 1) for a, b in self.pairs))


def plain_pairs(n_pairs: int = 4096, seed: int = SEED_BASE + 1) -> PairWorkload:
    rng = np.random.default_rng(seed)
    pairs = []
    for _ in range(n_pairs):
        seqs = []
        for _ in range(2):
            s = random_bases(rng, int(rng.integers(200, 601)))
            amb = rng.random(len(s)) < 0.01
            s[amb] = AMBIG[rng.integers(0, len(AMBIG), int(amb.sum()))]
            seqs.append(with_gap(s))
        pairs.append((seqs[0], seqs[1]))
    return PairWorkload("plain_pairs_4096x200-600_linear", pairs, 1, 2, 0)


def affine_pairs(n_pairs: int = 65536, seed: int = SEED_BASE + 2) -> PairWorkload:
    rng = np.random.default_rng(seed)
    lens = np.clip(np.round(rng.lognormal(np.log(800), 0.8, n_pairs)), 50, 4000).astype(int)
    pairs = []
    for L in lens:
        a = random_bases(rng, int(L))
        b = mutate(rng, a, 0.10, 0.02)
        if len(b) == 0:
            b = random_bases(rng, 1)
        pairs.append((with_gap(a), with_gap(b)))
    return PairWorkload(f"affine_pairs_{n_pairs}_lognormal800", pairs, 1, 1, 3)


def long_pairs(n_pairs: int = 512, seed: int = SEED_BASE + 5) -> PairWorkload:
    rng = np.random.default_rng(seed)
    pairs = []
    for _ in range(n_pairs):
        a = random_bases(rng, int(rng.integers(20000, 50001)))
        b = mutate(rng, a, 0.15, 0.02)
        pairs.append((with_gap(a), with_gap(b)))
    return PairWorkload(f"long_pairs_{n_pairs}x20-50kb_linear", pairs, 1, 2, 0)


def serving_pairs(n_pairs: int, seed: int = SEED_BASE + 4) -> PairWorkload:
    """Pairs with the serving workload's length/divergence distribution."""
    rng = np.random.default_rng(seed)
    lens = np.clip(np.round(rng.lognormal(np.log(1000), 0.8, n_pairs)), 100, 5000).astype(int)
    pairs = []
    for L in lens:
        a = random_bases(rng, int(L))
        b = mutate(rng, a, 0.25, 0.05)
        if len(b) == 0:
            b = random_bases(rng, 1)
        pairs.append((with_gap(a), with_gap(b)))
    return PairWorkload(f"serving_pairs_{n_pairs}", pairs, 1, 1, 3)


@dataclass
class TreeWorkload:
    """A rooted binary tree with sequences at the leaves.

    Leaves are 0..n-1; internal node k has children ``left[k]``, ``right[k]``
    (leaf index, or n + internal index), children before parents, and the
    last internal node is the root.
    """
    name: str
    leaves: list         # bitset sequences with leading gap
    left: np.ndarray
    right: np.ndarray
    subs: int
    indel: int
    gap_open: int

    @property
    def affine(self) -> bool:
        return self.gap_open > 0


def jc69_change(t: float) -> float:
    """Jukes-Cantor probability that a site differs after branch length t."""
    return 0.75 * (1.0 - np.exp(-4.0 * t / 3.0))


def yule_tree(n_taxa: int = 256, root_len: int = 1500, mean_branch: float = 0.05,
              indel_ratio: float = 0.2, seed: int = SEED_BASE + 3) -> TreeWorkload:
    """Yule topology, exponential branch lengths, sequences evolved from a
    uniform random root by JC69 substitutions and indels at indel_ratio x
    the substitution rate (geometric lengths, mean 3)."""
    rng = np.random.default_rng(seed)
    # grow the topology: split a uniformly chosen tip until n_taxa tips
    children = {0: None}
    tips = [0]
    nxt = 1
    while len(tips) < n_taxa:
        v = tips.pop(int(rng.integers(0, len(tips))))
        children[v] = (nxt, nxt + 1)
        children[nxt] = children[nxt + 1] = None
        tips += [nxt, nxt + 1]
        nxt += 2
    seq = {0: random_bases(rng, root_len)}
    order = [0]
    for v in order:  # parents before children
        if children[v] is None:
            continue
        for ch in children[v]:
            t = rng.exponential(mean_branch)
            s = substitute(rng, seq[v], jc69_change(t))
            seq[ch] = indels(rng, s, indel_ratio * t) if len(s) else s
            order.append(ch)
    # number leaves 0..n-1 and internal nodes in post-order
    leaf_id, int_id, left, right, leaves = {}, {}, [], [], []

    def visit(v):
        stack = [(v, False)]
        while stack:
            u, done = stack.pop()
            if children[u] is None:
                leaf_id[u] = len(leaves)
                s = seq[u] if len(seq[u]) else random_bases(rng, 1)
                leaves.append(with_gap(s))
            elif done:
                a, b = children[u]
                ref = lambda w: leaf_id[w] if w in leaf_id else n_taxa + int_id[w]
                int_id[u] = len(left)
                left.append(ref(a))
                right.append(ref(b))
            else:
                stack.append((u, True))
                a, b = children[u]
                stack.append((b, False))
                stack.append((a, False))

    visit(0)
    return TreeWorkload(f"yule_tree_{n_taxa}_root{root_len}", leaves,
                        np.array(left, np.int32), np.array(right, np.int32), 1, 2, 0)


@dataclass
class TripleWorkload:
    name: str
    triples: list        # [(s1, s2, p)] bitset sequences with leading gap
    mm: int
    go: int
    ge: int


def readjust_triples(n_triples: int = 2048, seed: int = SEED_BASE + 6, lo: int = 100,
                     hi: int = 300, sub_rate: float = 0.03,
                     indel_rate: float = 0.005) -> TripleWorkload:
    """Three-sequence readjustment inputs (Sequence.Align.readjust_3d: two
    children and a parent): a uniform ancestor of length U[lo, hi] and three
    descendants, each with `sub_rate` substitutions and indel events at
    `indel_rate` per site (geometric lengths, mean 2), 1% of positions an
    IUPAC ambiguity; costs as align_3_powell_inter takes them from POY's
    default linear matrix (mismatch 1, gap opening 0, gap 2)."""
    rng = np.random.default_rng(seed)
    triples = []
    for _ in range(n_triples):
        anc = random_bases(rng, int(rng.integers(lo, hi + 1)))
        t = []
        for _ in range(3):
            s = mutate(rng, anc, sub_rate, indel_rate, 2.0)
            if len(s) == 0:
                s = random_bases(rng, 1)
            amb = rng.random(len(s)) < 0.01
            s[amb] = AMBIG[rng.integers(0, len(AMBIG), int(amb.sum()))]
            t.append(with_gap(s))
        triples.append(tuple(t))
    return TripleWorkload(f"readjust_triples_{n_triples}x{lo}-{hi}_linear", triples, 1, 0, 2)
