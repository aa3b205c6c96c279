"""Seeded synthetic pair workloads with the shapes of the dCNS benchmark configurations.

Sequences are generated as text (upper-case ACGT, with masked runs written as lower-case 'n' the way dCNS's k-mer
masking marks them), then encoded exactly as the cut1Gap driver does before calling the pair aligner:
lower-case 'n' is deleted (controlLayer4.cpp:1387,1406 of the reference) and the rest is mapped by
SequenceCharToUInt8 (impl/SequenceCharToUInt8.cpp:6-33): A/a=0, C/c=1, G/g=3, T/t/U/u=4, anything else=2.
"""
from __future__ import annotations

import numpy as np

_LUT = np.full(256, 2, dtype=np.int8)
for _c, _v in (("A", 0), ("C", 1), ("G", 3), ("T", 4), ("U", 4)):
    _LUT[ord(_c)] = _v
    _LUT[ord(_c.lower())] = _v

_BASES = np.frombuffer(b"ACGT", dtype=np.uint8)


def encode(seq: str) -> np.ndarray:
    """dCNS integer codes of a sequence whose lower-case 'n' runs were already removed."""
    return _LUT[np.frombuffer(seq.encode(), dtype=np.uint8)]


def strip_masked(seq: str) -> str:
    return seq.replace("n", "")


def prepare(seq: str) -> np.ndarray:
    return encode(strip_masked(seq))


def random_seq(rng: np.random.Generator, n: int, gc: float = 0.5) -> bytearray:
    p = np.array([(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2])
    return bytearray(_BASES[rng.choice(4, size=n, p=p)].tobytes())


def mutate(rng, seg: bytes, identity: float, indel_rate: float) -> bytes:
    """Uniform substitutions to `identity`, then 1-5 bp insertions/deletions starting at rate `indel_rate`."""
    arr = np.frombuffer(seg, dtype=np.uint8).copy()
    n = len(arr)
    sub = rng.random(n) > identity
    if sub.any():
        idx = np.searchsorted(_BASES, arr[sub])
        arr[sub] = _BASES[(idx + rng.integers(1, 4, int(sub.sum()))) % 4]
    if indel_rate <= 0:
        return arr.tobytes()
    parts, prev = [], 0
    for p in np.nonzero(rng.random(n) < indel_rate)[0]:
        if p < prev:
            continue
        parts.append(arr[prev:p].tobytes())
        k = int(rng.integers(1, 6))
        if rng.random() < 0.5:
            prev = int(p) + k  # deletion
        else:
            parts.append(bytes(random_seq(rng, k)))  # insertion
            prev = int(p)
    parts.append(arr[prev:].tobytes())
    return b"".join(parts)


def mask_runs(rng, seq: bytearray, frac: float, lo: int, hi: int, soft: bool = False) -> None:
    """Mask about `frac` of the sequence in runs of lo..hi bp: 'n' (hard, deleted before alignment) or lower case."""
    n = len(seq)
    arr = np.frombuffer(seq, dtype=np.uint8).copy()
    upper = np.isin(arr, _BASES)
    target = int(frac * n)
    done = 0
    for _ in range(10000):
        if done >= target:
            break
        L = int(rng.integers(lo, hi + 1))
        s = int(rng.integers(0, max(1, n - L)))
        m = upper[s:s + L]
        done += int(m.sum())
        seg = arr[s:s + L]
        seg[m] = (seg[m] + 32) if soft else ord("n")
        upper[s:s + L] = False
    seq[:] = arr.tobytes()


def planted_pair(rng, n1: int, n2: int, nseg: int, seg_lo: int, seg_hi: int, id_lo: float, id_hi: float,
                 indel: float, mask_frac: float, mask_lo: int = 20, mask_hi: int = 500, gc: float = 0.5,
                 soft_mask: bool = False, dup_blocks: int = 0):
    """Reference/query text pair with `nseg` conserved segments copied from the reference into the query at the same
    relative position, mutated to a uniform identity in [id_lo, id_hi] with 1-5 bp indels at rate `indel`."""
    a = random_seq(rng, n1, gc)
    b = random_seq(rng, n2, gc)
    for _ in range(nseg):
        L = int(rng.integers(seg_lo, seg_hi + 1))
        if L >= n1 or L >= n2:
            continue
        s1 = int(rng.integers(0, n1 - L))
        s2 = min(int(s1 / n1 * n2), n2 - L)
        ident = float(rng.uniform(id_lo, id_hi))
        seg = mutate(rng, bytes(a[s1:s1 + L]), ident, indel)[:n2 - s2]
        b[s2:s2 + len(seg)] = seg
    for _ in range(dup_blocks):  # transposon-like duplicated blocks inserted into the query
        L = int(rng.integers(2000, 10001))
        if L >= n1:
            continue
        s1 = int(rng.integers(0, n1 - L))
        pos = int(rng.integers(0, len(b)))
        b[pos:pos] = mutate(rng, bytes(a[s1:s1 + L]), 0.9, 0.01)
    if mask_frac > 0:
        mask_runs(rng, a, mask_frac, mask_lo, mask_hi, soft_mask)
        mask_runs(rng, b, mask_frac, mask_lo, mask_hi, soft_mask)
    return a.decode(), b.decode()


def single_pair_5kb(seed: int = 20261204):
    """One 5,000 x 5,000 pair, 20 planted 30-200 bp segments at 85 % identity, 1 % indels, 20 % 'n'-masked in runs of
    20-500 bp.  Returns [(seq1 codes, seq2 codes)]."""
    rng = np.random.default_rng(seed)
    a, b = planted_pair(rng, 5000, 5000, 20, 30, 200, 0.85, 0.85, 0.01, 0.20)
    return [(prepare(a), prepare(b))]


def lognormal_lengths(rng, n, median, sigma, lo, hi):
    return np.clip(np.round(rng.lognormal(np.log(median), sigma, size=n)), lo, hi).astype(int)


def batched_pairs(n_pairs: int = 10000, seed: int = 20261205, sigma: float = 0.8):
    """Batched workload: independent pairs with log-normal lengths (median 3 kb, clipped to 0.5-20 kb) drawn
    independently for both sequences, Poisson(8) planted segments capped at 30, 30-300 bp, identity U(70,95)%,
    1 % indels, 15 % masked runs.  sigma=0.8 is this project's choice (the benchmark fixes only the median/clip)."""
    rng = np.random.default_rng(seed)
    n1 = lognormal_lengths(rng, n_pairs, 3000, sigma, 500, 20000)
    n2 = lognormal_lengths(rng, n_pairs, 3000, sigma, 500, 20000)
    out = []
    for k in range(n_pairs):
        nseg = min(int(rng.poisson(8)), 30)
        a, b = planted_pair(rng, int(n1[k]), int(n2[k]), nseg, 30, 300, 0.70, 0.95, 0.01, 0.15)
        out.append((prepare(a), prepare(b)))
    return out


def long_pairs_200kb(n_pairs: int = 64, length: int = 200000, seed: int = 20261206):
    """Long pairs: 200 kb x 200 kb at GC 45 %, 500 planted 20-400 bp segments at 80 % identity, and 5 duplicated
    2-10 kb blocks inserted into the query."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_pairs):
        a, b = planted_pair(rng, length, length, 500, 20, 400, 0.80, 0.80, 0.01, 0.0, gc=0.45, dup_blocks=5)
        out.append((prepare(a), prepare(b)))
    return out


def extension_seeds(n_seeds: int = 1000000, seed: int = 20261207):
    """Extension stress: per seed, a 38 bp core with 0-7 substitutions (SW score 41-76 at the default scoring) followed
    by flanks of U(50, 2000) bp whose query copy has identity U(50, 98) % and 1-5 bp indels at rate U(0, 3) %.
    Returns [(seq1 codes, seq2 codes)], each pair starting at the seed as x_extend_seed's forward pass sees it."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_seeds):
        core = random_seq(rng, 38)
        core2 = bytearray(core)
        for pos in rng.choice(38, size=int(rng.integers(0, 8)), replace=False):
            k = int(np.searchsorted(_BASES, core2[pos]))
            core2[pos] = int(_BASES[(k + int(rng.integers(1, 4))) % 4])
        flank = random_seq(rng, int(rng.integers(50, 2001)))
        flank2 = mutate(rng, bytes(flank), float(rng.uniform(0.50, 0.98)), float(rng.uniform(0.0, 0.03)))
        out.append((encode((core + flank).decode()), encode((core2 + flank2).decode())))
    return out


def serving_requests(n_requests: int = 2000, seed: int = 20261208, long_frac: float = 0.10):
    """Serving requests: lengths log-normal (median 4 kb, sigma 1.0) clipped to 200 bp-100 kb, drawn independently for
    both sequences, except that a `long_frac` share of the requests (chosen at random) draws both from U(50, 100] kb:
    the log-normal alone puts well under 1 % above 50 kb, and the serving configuration fixes 10 %.  Planted 30-300 bp
    segments at U(70, 95) % identity, Poisson(8) per 3 kb of the shorter sequence (capped at 300), 1 % indels, 15 %
    masked runs.  Arrival times are drawn by the caller (a Poisson process at the configured rate)."""
    rng = np.random.default_rng(seed)
    n1 = lognormal_lengths(rng, n_requests, 4000, 1.0, 200, 100000)
    n2 = lognormal_lengths(rng, n_requests, 4000, 1.0, 200, 100000)
    long = rng.random(n_requests) < long_frac
    n1[long] = rng.integers(50001, 100001, int(long.sum()))
    n2[long] = rng.integers(50001, 100001, int(long.sum()))
    out = []
    for k in range(n_requests):
        nseg = min(int(rng.poisson(8.0 * min(n1[k], n2[k]) / 3000.0)), 300)
        a, b = planted_pair(rng, int(n1[k]), int(n2[k]), nseg, 30, 300, 0.70, 0.95, 0.01, 0.15)
        out.append((prepare(a), prepare(b)))
    return out


def random_pair(rng, n1, n2, alphabet=5):
    """Uniform codes over {0..alphabet-1} (alphabet=5 includes N=2) for exhaustive/edge tests."""
    return (rng.integers(0, alphabet, size=n1).astype(np.int8), rng.integers(0, alphabet, size=n2).astype(np.int8))
