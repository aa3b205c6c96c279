"""Generates tests/golden/seeded_chromosome.npz: cut2Gaps2's seeded 2-gap overload (findSimilarFragmentsForPairedSequence
with maximumAlignLength, impl/findSimilarFragmentsForPairedSequence4.cpp:624-745) on a whole 200 kb x ~234 kb pair of
the long-pair workload, past the 140 kb that the reference's driver caps it at (controlLayer4.cpp:1816: its dense
(max+1)^2-byte traceback matrix).  Computed by the reference, unmodified except for that matrix
(oracle/_ref/libdcns_ref_lazy.so: oracle/lazy_matrix.cpp keeps its get/set/reset semantics and stores only the touched
cells), with maximumAlignLength 250,000 (no cap for this pair), and by the oracle restatement without a cap; the two
must agree.  Run here, where the reference exists (about an hour of one core):

    python tests/golden/make_seeded_chromosome.py

The x-seeds are 0-based (start1, end1, start2, end2) quadruples: the first 16 cut1Gap fragments of the whole pair (as
cut2Gaps2 reads them from a SAM file of earlier alignments), then the first two again shifted a few bases to also
exercise the overload's cover test and seed handling, in that order.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

N_SEEDS, REF_CAP = 16, 250000


def case():
    from dcns_gb300 import workloads as W
    from oracle import oracle as O
    a, b = W.long_pairs_200kb(n_pairs=1)[0]
    frs = O.Oracle().find(a, b)[0][:N_SEEDS]
    seeds = [(f.start1 - 1, f.end1 - 1, f.start2 - 1, f.end2 - 1) for f in frs]
    seeds += [(s1 + 3, e1 - 2, s2 + 3, e2 - 2) for s1, e1, s2, e2 in seeds[:2]]
    return a, b, seeds


def main():
    from oracle import oracle as O
    import digest as D
    O.build()
    t0 = time.time()
    a, b, seeds = case()
    print(f"{len(seeds)} seeds, {time.time() - t0:.0f} s", flush=True)
    got = O.Oracle().find_seeded(a, b, seeds, 1 << 30)
    print(f"oracle: {len(got)} fragments, {time.time() - t0:.0f} s", flush=True)
    ref = O.Reference(lazy=True).find_seeded(a, b, seeds, REF_CAP)
    print(f"reference: {len(ref)} fragments, {time.time() - t0:.0f} s", flush=True)
    assert [f.key() for f in got] == [f.key() for f in ref], "oracle and reference differ"
    for x, y in zip(got, ref):
        assert abs(x.pvalue - y.pvalue) <= 1e-12 * max(1.0, abs(y.pvalue))
    frag = np.array([[f.start1, f.end1, f.start2, f.end2, f.score] for f in ref], np.int64).reshape(-1, 5)
    cg = [np.asarray(f.cigar, np.uint32) for f in ref]
    off = np.cumsum([0] + [len(c) for c in cg]).astype(np.int64)
    dst = os.path.join(HERE, "seeded_chromosome.npz")
    np.savez_compressed(dst, seeds=np.array(seeds, np.int32), frag=frag,
                        cigar=np.concatenate(cg) if cg else np.zeros(0, np.uint32), cigar_off=off,
                        pe=np.array([[f.pvalue, f.evalue] for f in ref], np.float64).reshape(-1, 2),
                        inputs=np.array(D.inputs_hash([(a, b)])))
    print("wrote", dst, os.path.getsize(dst), "bytes;", len(ref), "fragments;", f"{time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()
