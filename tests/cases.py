"""Seeded test inputs shared by the CPU and GPU parity tests."""
from __future__ import annotations

import numpy as np

GAP = 16
STD_TCM = [[0 if r == c else (2 if (r == 4 or c == 4) else 1) for c in range(5)]
           for r in range(5)]
AFF_TCM = [[0 if r == c else 1 for c in range(5)] for r in range(5)]  # subs 1, ext 1


def rseq(rng, n, amb=0.0, gapp=0.0):
    s = rng.choice(np.array([1, 2, 4, 8], np.uint8), size=n)
    if amb:
        m = rng.random(n) < amb
        s[m] = rng.integers(1, 16, int(m.sum()))
    if gapp:
        m = rng.random(n) < gapp
        s[m] = s[m] | 16
    return np.concatenate([[GAP], s]).astype(np.uint8)


def mutate(rng, s, sub=0.1, ind=0.05):
    out = [GAP]
    for x in s[1:]:
        r = rng.random()
        if r < ind / 2:
            continue
        if r < ind:
            out.extend(int(rng.choice([1, 2, 4, 8])) for _ in range(int(rng.geometric(1 / 3))))
        out.append(int(rng.choice([1, 2, 4, 8])) if rng.random() < sub else int(x))
    return np.array(out, np.uint8)


def edge_pairs():
    """Hand-made cases: identity, single edits, ambiguity, gap-bearing states,
    the shortest inputs, and both argument orders."""
    enc = {"A": 1, "C": 2, "G": 4, "T": 8, "R": 5, "N": 15, "-": 16, "a": 17, "c": 18}
    S = lambda t: np.array([GAP] + [enc[ch] for ch in t], np.uint8)
    base = [
        ("ACGTACGT", "ACGTACGT"), ("ACGTACGT", "ACGAACGT"), ("ACGTACGT", "ACGTCGT"),
        ("A", "R"), ("A", "C"), ("", "ACGT"), ("A", "A"), ("ACGT", ""),
        ("ACGTTTTTACG", "ACGACG"), ("NNNN", "ACGT"), ("AaCcG", "ACG"),
        ("ACGT" * 30, "ACGT" * 29 + "AC"), ("A" * 50, "C" * 50), ("A" * 5, "A" * 90),
        ("ACGTACGTAC" * 3, "TTTT"), ("GATTACA", "GCATGCT"),
    ]
    out = []
    for a, b in base:
        out.append((S(a), S(b)))
        out.append((S(b), S(a)))
    return out


def random_pairs(rng, n, maxlen=300, kinds=5):
    pairs = []
    for t in range(n):
        L = int(rng.choice([5, 30, 100, maxlen]))
        n1 = int(rng.integers(1, L))
        kind = t % kinds
        a = rseq(rng, n1, amb=0.05 if kind == 1 else 0, gapp=0.15 if kind == 2 else 0)
        b = mutate(rng, a, 0.15, 0.06) if kind != 3 else rseq(rng, int(rng.integers(1, L)))
        if len(a) == 1 and len(b) == 1:
            continue
        if rng.random() < 0.5:
            a, b = b, a
        pairs.append((a, b))
    return pairs
