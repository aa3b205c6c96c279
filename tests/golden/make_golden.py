"""Generates tests/golden/golden.npz from the UNMODIFIED dCNS reference (oracle/_ref/libdcns_ref.so, built from the
reference checkout by oracle/build_ref.sh).  Run here, where the reference exists:

    python tests/golden/make_golden.py [/path/to/reference]

Inputs are seeded synthetic sequences plus the inline sequences of the reference's own test
test/impl/smithWaterman.cpp (read from that file as text at generation time).  Every expected value is what the
reference computed; nothing is derived from the restatement.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from dcns_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


class Packer:
    """Ragged int arrays -> one flat array + offsets."""

    def __init__(self, dtype):
        self.parts, self.dtype = [], dtype

    def add(self, a):
        self.parts.append(np.asarray(a, dtype=self.dtype))

    def arrays(self):
        off = np.zeros(len(self.parts) + 1, np.int64)
        off[1:] = np.cumsum([len(p) for p in self.parts])
        flat = np.concatenate(self.parts) if self.parts else np.zeros(0, self.dtype)
        return flat, off


def inline_test_sequences(refdir):
    """The active (non-commented) seq1/seq2 literals of the reference's smithWaterman test, per TEST block."""
    path = os.path.join(refdir, "test", "impl", "smithWaterman.cpp")
    text = open(path).read()
    pairs = []
    for block in re.split(r"\nTEST\(", text)[1:]:
        s1 = re.search(r'^\s*std::string seq1_string\s*=\s*"([A-Za-z]+)"', block, re.M)
        s2 = re.search(r'^\s*std::string seq2_string\s*=\s*"([A-Za-z]+)"', block, re.M)
        if s1 and s2:
            pairs.append((s1.group(1), s2.group(1)))
    return pairs


def main(refdir):
    ref = O.Reference()
    rng = np.random.default_rng(20261203)
    out = {}

    # ---- known-answer cases from the reference's own test inputs
    inline = inline_test_sequences(refdir)
    assert len(inline) >= 2, "expected two active sequence pairs in test/impl/smithWaterman.cpp"
    ka_a, ka_b = Packer(np.int8), Packer(np.int8)
    ka_sw, ka_xe, ka_sg = [], [], []
    ka_cg = Packer(np.uint32)
    for s1, s2 in inline[:2]:
        a, b = W.encode(s1), W.encode(s2)
        ka_a.add(a)
        ka_b.add(b)
        ka_sw.append(ref.sw(a, b))
        x = ref.xextend(a, b, cigar=True)
        ka_xe.append((x["score"], x["end1"], x["end2"], x["iii"], x["jjj"]))
        ka_cg.add(x["cigar"])
        # the reference test's 2-piece parameters (test/impl/smithWaterman.cpp:94-102)
        g = ref.semiglobal(a, b, cigar=True, open2=-80, ext2=-1, zdrop=100, bandwidth=100)
        ka_sg.append((g["score"], g["end1"], g["end2"]))
        ka_cg.add(g["cigar"])
    out["ka_a"], out["ka_a_off"] = ka_a.arrays()
    out["ka_b"], out["ka_b_off"] = ka_b.arrays()
    out["ka_sw"] = np.array(ka_sw, np.int32)
    out["ka_xe"] = np.array(ka_xe, np.int32)
    out["ka_sg"] = np.array(ka_sg, np.int32)
    out["ka_cigar"], out["ka_cigar_off"] = ka_cg.arrays()

    # ---- seed-scan Smith-Waterman: random (with N), planted, and exhaustive tiny cases
    A, B = Packer(np.int8), Packer(np.int8)
    exp, prm = [], []
    for t in range(600):
        n1, n2 = int(rng.integers(0, 200)), int(rng.integers(0, 70))
        a, b = W.random_pair(rng, n1, n2, alphabet=int(rng.choice([2, 4, 5])))
        p = (-4, -2, 2, -3) if t % 4 else (int(rng.integers(-8, -1)), int(rng.integers(-3, 0)), int(rng.integers(1, 4)),
                                          int(rng.integers(-4, 0)))
        A.add(a), B.add(b)
        exp.append(ref.sw(a, b, *p))
        prm.append(p)
    for t in range(200):
        x, y = W.planted_pair(rng, int(rng.integers(60, 600)), 38, 1, 30, 38, 0.7, 1.0, 0.03, 0.0)
        a, b = W.prepare(x), W.prepare(y)
        A.add(a), B.add(b)
        exp.append(ref.sw(a, b))
        prm.append((-4, -2, 2, -3))
    for n1 in range(0, 6):  # every pair of lengths <= 5 over {A, C, N} plus T on the longer side
        for n2 in range(0, 5):
            for k in range(20):
                a, b = W.random_pair(rng, n1, n2)
                A.add(a), B.add(b)
                exp.append(ref.sw(a, b))
                prm.append((-4, -2, 2, -3))
    out["sw_a"], out["sw_a_off"] = A.arrays()
    out["sw_b"], out["sw_b_off"] = B.arrays()
    out["sw_exp"] = np.array(exp, np.int32)
    out["sw_prm"] = np.array(prm, np.int32)

    # ---- x-drop extension with and without cigar, various w / xdrop
    A, B, CG = Packer(np.int8), Packer(np.int8), Packer(np.uint32)
    exp, prm = [], []
    for t in range(400):
        if t % 2:
            x, y = W.planted_pair(rng, int(rng.integers(20, 400)), int(rng.integers(20, 400)), 1, 20, 300, 0.6, 1.0,
                                  0.03, 0.0)
            a, b = W.prepare(x), W.prepare(y)
        else:
            a, b = W.random_pair(rng, int(rng.integers(1, 300)), int(rng.integers(1, 300)),
                                 alphabet=int(rng.choice([2, 4, 5])))
        w = int(rng.choice([10, 10, 10, 3, 1]))
        xd = int(rng.choice([20, 20, 5, 50]))
        cig = bool(t % 3)
        r = ref.xextend(a, b, xdrop=xd, w=w, cigar=cig)
        A.add(a), B.add(b), CG.add(r["cigar"])
        exp.append((r["score"], r["end1"], r["end2"], r["iii"], r["jjj"]))
        prm.append((w, xd, int(cig)))
    out["xe_a"], out["xe_a_off"] = A.arrays()
    out["xe_b"], out["xe_b_off"] = B.arrays()
    out["xe_cigar"], out["xe_cigar_off"] = CG.arrays()
    out["xe_exp"] = np.array(exp, np.int32)
    out["xe_prm"] = np.array(prm, np.int32)

    # ---- 2-piece semi-global with and without cigar
    A, B, CG = Packer(np.int8), Packer(np.int8), Packer(np.uint32)
    exp, prm = [], []
    for t in range(300):
        if t % 2:
            x, y = W.planted_pair(rng, int(rng.integers(20, 300)), int(rng.integers(20, 300)), 2, 20, 150, 0.6, 1.0,
                                  0.03, 0.0)
            a, b = W.prepare(x), W.prepare(y)
        else:
            a, b = W.random_pair(rng, int(rng.integers(1, 250)), int(rng.integers(1, 250)),
                                 alphabet=int(rng.choice([2, 4, 5])))
        bw = int(rng.choice([20000, 20000, 100, 10, 2]))
        zd = int(rng.choice([50, 50, 100, 10]))
        o2, e2 = [(-45, 0), (-45, 0), (-80, -1), (-20, -1)][t % 4]
        cig = bool(t % 3)
        r = ref.semiglobal(a, b, cigar=cig, bandwidth=bw, zdrop=zd, open2=o2, ext2=e2)
        A.add(a), B.add(b), CG.add(r["cigar"])
        exp.append((r["score"], r["end1"], r["end2"]))
        prm.append((bw, zd, o2, e2, int(cig)))
    out["sg_a"], out["sg_a_off"] = A.arrays()
    out["sg_b"], out["sg_b_off"] = B.arrays()
    out["sg_cigar"], out["sg_cigar_off"] = CG.arrays()
    out["sg_exp"] = np.array(exp, np.int32)
    out["sg_prm"] = np.array(prm, np.int32)

    # ---- whole pipelines: the config-1 pair plus small planted pairs (1-gap and 2-gap)
    pairs = list(W.single_pair_5kb())
    for t in range(24):
        n1, n2 = int(rng.integers(40, 2500)), int(rng.integers(8, 2500))
        x, y = W.planted_pair(rng, n1, n2, int(rng.integers(0, 10)), 30, 300, 0.7, 0.98, 0.01,
                              float(rng.choice([0.0, 0.15])), soft_mask=bool(t % 5 == 0))
        pairs.append((W.prepare(x), W.prepare(y)))
    A, B = Packer(np.int8), Packer(np.int8)
    for gap, name in ((False, "p1"), (True, "p2")):
        F, PE, CG, NF = [], [], Packer(np.uint32), []
        for a, b in pairs:
            fr = ref.find(a, b, two_gap=gap)
            NF.append(len(fr))
            for f in fr:
                F.append((f.start1, f.end1, f.start2, f.end2, f.score))
                PE.append((f.pvalue, f.evalue))
                CG.add(f.cigar)
        out[name + "_frag"] = np.array(F, np.int64).reshape(-1, 5)
        out[name + "_pe"] = np.array(PE, np.float64).reshape(-1, 2)
        out[name + "_cigar"], out[name + "_cigar_off"] = CG.arrays()
        out[name + "_nfrag"] = np.array(NF, np.int64)
    RAW, LNK, NR, NL = [], [], [], []
    for a, b in pairs:
        A.add(a), B.add(b)
        raw, lk = ref.seeds(a, b)
        RAW += raw
        LNK += lk
        NR.append(len(raw))
        NL.append(len(lk))
    out["pp_a"], out["pp_a_off"] = A.arrays()
    out["pp_b"], out["pp_b_off"] = B.arrays()
    out["seeds_raw"] = np.array(RAW, np.int32).reshape(-1, 4)
    out["seeds_linked"] = np.array(LNK, np.int32).reshape(-1, 4)
    out["seeds_nraw"] = np.array(NR, np.int64)
    out["seeds_nlinked"] = np.array(NL, np.int64)

    # ---- slidingWindowAlignment text output for 3 sequences (reference = first)
    seqs = [W.prepare(s) for s in W.planted_pair(rng, 700, 900, 4, 30, 120, 0.8, 0.95, 0.01, 0.0)]
    seqs.append(W.random_pair(rng, 300, 1)[0])
    rows = ref.sliding(seqs)
    S = Packer(np.int8)
    for s in seqs:
        S.add(s)
    out["sl_seq"], out["sl_seq_off"] = S.arrays()
    out["sl_rows"] = np.array([(j, i) for j, i, _ in rows], np.int64)
    out["sl_text"] = np.array([s for _, _, s in rows])

    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes;", len(pairs), "pipeline pairs,",
          int(out["p1_nfrag"].sum()), "1-gap and", int(out["p2_nfrag"].sum()), "2-gap fragments")


if __name__ == "__main__":
    refdir = sys.argv[1] if len(sys.argv) > 1 else O.reference_dir()
    O.build()
    main(refdir)
