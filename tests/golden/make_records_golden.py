"""Generates tests/golden/records.npz: SAM and "o" text written by the UNMODIFIED dCNS reference's own outputMasking
(controlLayer4.cpp:835-1358, through oracle/_ref/libdcns_ref_cli.so built by oracle/build_ref.sh) for fragments the
reference computed on seeded masked pairs, under all four strand combinations.  Run here, where the reference exists:

    python tests/golden/make_records_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from dcns_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

CLI = os.path.join(ROOT, "oracle", "_ref", "libdcns_ref_cli.so")
STRANDS = [(1, 1), (1, 0), (0, 1), (0, 0)]


def cases():
    """(ref_text, qry_text) region texts with 'n' runs (hard masking) or lower-case runs (soft masking); short runs
    land inside conserved segments, so CIGARs cross masked stretches."""
    out = []
    for k, (n1, n2, soft, frac, lo, hi) in enumerate([(3000, 3200, False, 0.20, 20, 500), (5000, 5000, False, 0.20, 20, 500),
                                                     (2500, 2000, True, 0.20, 20, 500), (4000, 3600, False, 0.30, 5, 40),
                                                     (6000, 6500, False, 0.25, 3, 25), (3500, 3500, False, 0.0, 20, 20)]):
        rng = np.random.default_rng(9100 + k)
        a, b = W.planted_pair(rng, n1, n2, 30, 40, 300, 0.88, 0.98, 0.01, frac, mask_lo=lo, mask_hi=hi,
                              soft_mask=soft)
        out.append((a, b))
    return out


def flatten(frs):
    n = len(frs)
    frag = np.zeros((max(n, 1), 7), np.int64)
    cig, pv, ev = [], np.zeros(max(n, 1)), np.zeros(max(n, 1))
    for k, f in enumerate(frs):
        frag[k, :5] = (f.start1, f.end1, f.start2, f.end2, f.score)
        frag[k, 5], frag[k, 6] = len(cig), len(f.cigar)
        cig.extend(f.cigar)
        pv[k], ev[k] = f.pvalue, f.evalue
    return frag, np.asarray(cig if cig else [0], np.uint32), pv, ev


def reference_records(lib, frs, t1, t2, rs, qs, r0, q0, rchr, qchr):
    frag, cg, pv, ev = flatten(frs)
    with tempfile.TemporaryDirectory() as d:
        prefix = os.path.join(d, "out")
        P = C.POINTER
        rc = lib.ref_output_masking(prefix.encode(), C.c_int64(len(frs)), frag.ctypes.data_as(P(C.c_int64)),
                                    cg.ctypes.data_as(P(C.c_uint32)), pv.ctypes.data_as(P(C.c_double)),
                                    ev.ctypes.data_as(P(C.c_double)), rs, qs, C.c_int32(r0), C.c_int32(q0),
                                    rchr.encode(), qchr.encode(), t1.encode(), C.c_int64(len(t1)), t2.encode(),
                                    C.c_int64(len(t2)))
        assert rc == 0
        with open(prefix + ".sam") as f:
            sam = f.read()
        with open(prefix + "o") as f:
            o = f.read()
    return sam, o


def ragged(items, dtype):
    off = np.zeros(len(items) + 1, np.int64)
    off[1:] = np.cumsum([len(x) for x in items])
    flat = np.concatenate([np.asarray(x, dtype) for x in items]) if items else np.zeros(0, dtype)
    return flat, off


def main():
    lib = C.CDLL(CLI)
    orc = O.Reference()
    texts, frag_rows, cig, pvev, case_off, rows, sams, os_ = [], [], [], [], [0], [], [], []
    for ci, (t1, t2) in enumerate(cases()):
        texts += [np.frombuffer(t1.encode(), np.uint8), np.frombuffer(t2.encode(), np.uint8)]
        frs = orc.find(W.prepare(t1), W.prepare(t2))
        for f in frs:
            frag_rows.append((f.start1, f.end1, f.start2, f.end2, f.score, len(cig), len(f.cigar)))
            cig.extend(f.cigar)
            pvev.append((f.pvalue, f.evalue))
        case_off.append(len(frag_rows))
        for rs, qs in STRANDS:
            r0, q0 = 1000 * (ci + 1) + 17, 2000 * (ci + 1) + 3
            sam, o = reference_records(lib, frs, t1, t2, rs, qs, r0, q0, f"chr{ci + 1}", f"scaffold_{ci}")
            rows.append((ci, rs, qs, r0, q0))
            sams.append(np.frombuffer(sam.encode(), np.uint8))
            os_.append(np.frombuffer(o.encode(), np.uint8))
    tx, tx_off = ragged(texts, np.uint8)
    sm, sm_off = ragged(sams, np.uint8)
    oo, oo_off = ragged(os_, np.uint8)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "records.npz"), texts=tx, texts_off=tx_off,
                        frags=np.array(frag_rows, np.int64).reshape(-1, 7), cigar=np.array(cig, np.uint32),
                        pvev=np.array(pvev, np.float64).reshape(-1, 2), case_off=np.array(case_off, np.int64),
                        rows=np.array(rows, np.int64), sam=sm, sam_off=sm_off, o=oo, o_off=oo_off)
    print("records.npz:", len(rows), "record sets,", len(frag_rows), "fragments")


if __name__ == "__main__":
    main()
