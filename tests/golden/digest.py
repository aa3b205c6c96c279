"""Compact digests of whole-workload results, so that the outputs of the unmodified reference on the full benchmark
workloads fit in small fixtures: per pair the fragment count, a 64-bit BLAKE2b hash of every fragment's integer
fields and CIGAR words (in order), and the sums of the p- and e-values; per x-drop task its integer outputs and a hash
of its CIGAR.  The inputs are regenerated from their seeded generators, and a hash of them is stored beside the
digests so that a generator that draws differently on another machine is reported as such."""
from __future__ import annotations

import hashlib

import numpy as np


def fragments_hash(frags) -> int:
    h = hashlib.blake2b(digest_size=8)
    for f in frags:
        cg = np.asarray(list(f.cigar), np.uint32)
        h.update(np.array([f.start1, f.end1, f.start2, f.end2, f.score, len(cg)], np.int64).tobytes())
        h.update(cg.tobytes())
    return int.from_bytes(h.digest(), "little")


def cigar_hash(cigar) -> int:
    return int.from_bytes(hashlib.blake2b(np.asarray(list(cigar), np.uint32).tobytes(), digest_size=8).digest(),
                          "little")


def inputs_hash(pairs) -> str:
    h = hashlib.blake2b(digest_size=16)
    for a, b in pairs:
        h.update(np.array([len(a), len(b)], np.int64).tobytes())
        h.update(np.asarray(a, np.int8).tobytes())
        h.update(np.asarray(b, np.int8).tobytes())
    return h.hexdigest()


def pair_digests(results):
    """(nfrag int32 [n], hash uint64 [n], p/e sums float64 [n, 2]) of per-pair fragment lists."""
    n = len(results)
    nf = np.zeros(n, np.int32)
    hs = np.zeros(n, np.uint64)
    pe = np.zeros((n, 2), np.float64)
    for i, frs in enumerate(results):
        frs = list(frs)
        nf[i] = len(frs)
        hs[i] = fragments_hash(frs)
        pe[i] = (sum(f.pvalue for f in frs), sum(f.evalue for f in frs))
    return nf, hs, pe


def compare_pairs(got, exp_nf, exp_hs, exp_pe, rel=1e-12):
    """Indices of pairs whose fragments differ (count or hash), and of pairs whose p/e sums differ beyond `rel`."""
    nf, hs, pe = pair_digests(got)
    bad = np.nonzero((nf != exp_nf) | (hs != exp_hs))[0]
    tol = rel * np.maximum(np.abs(exp_pe), 1e-300)
    bad_pe = np.nonzero(np.any(np.abs(pe - exp_pe) > tol, axis=1))[0]
    return bad, bad_pe
