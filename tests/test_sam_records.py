"""SAM and "o" records as cut1Gap writes them (outputMasking), from the library's host formatter, byte for byte
against text the reference's own writer produced (committed fixture, and live when the reference builds here)."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

import dcns_gb300 as D

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "records.npz")


def _load():
    z = np.load(GOLD)
    texts = [bytes(z["texts"][z["texts_off"][k]:z["texts_off"][k + 1]]).decode() for k in range(len(z["texts_off"]) - 1)]
    frs_per_case = []
    for c in range(len(z["case_off"]) - 1):
        frs = []
        for r in range(z["case_off"][c], z["case_off"][c + 1]):
            f = z["frags"][r]
            frs.append(SimpleNamespace(start1=int(f[0]), end1=int(f[1]), start2=int(f[2]), end2=int(f[3]),
                                       score=int(f[4]), cigar=[int(x) for x in z["cigar"][f[5]:f[5] + f[6]]],
                                       pvalue=float(z["pvev"][r, 0]), evalue=float(z["pvev"][r, 1])))
        frs_per_case.append(frs)
    rows = []
    for k, (c, rs, qs, r0, q0) in enumerate(z["rows"]):
        sam = bytes(z["sam"][z["sam_off"][k]:z["sam_off"][k + 1]]).decode()
        o = bytes(z["o"][z["o_off"][k]:z["o_off"][k + 1]]).decode()
        rows.append((int(c), int(rs), int(qs), int(r0), int(q0), sam, o))
    return texts, frs_per_case, rows


def _built():
    try:
        D.library()
        return True
    except Exception:  # noqa: BLE001
        return False


pytestmark = pytest.mark.skipif(not _built(), reason="library not built")


def test_records_match_reference_writer_fixture():
    texts, frs_per_case, rows = _load()
    assert len(rows) == 24 and sum(len(f) for f in frs_per_case) > 50
    n_masked_ops = 0
    for c, rs, qs, r0, q0, sam, o in rows:
        got_sam, got_o = D.format_records(frs_per_case[c], texts[2 * c], texts[2 * c + 1], rs, qs, r0, q0,
                                          f"chr{c + 1}", f"scaffold_{c}")
        assert got_o == o, (c, rs, qs)
        assert got_sam == sam, (c, rs, qs)
        n_masked_ops += sum(1 for line in sam.splitlines() if "D" in line.split("\t")[5])
    assert n_masked_ops > 0


def test_records_live_reference_writer(tmp_path):
    """The same comparison on fresh fragments of the restatement, through the reference writer built here."""
    cli = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libdcns_ref_cli.so")
    if not os.path.exists(cli):
        pytest.skip("reference writer not built on this host")
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_records_golden as G
    from dcns_gb300 import workloads as W
    from oracle import oracle as O
    import ctypes as C

    lib = C.CDLL(cli)
    orc = O.Oracle()
    rng = np.random.default_rng(77)
    for k in range(3):
        a, b = W.planted_pair(rng, 3000 + 500 * k, 2800, 25, 40, 250, 0.9, 0.98, 0.01, 0.25, mask_lo=4, mask_hi=30)
        frs = orc.find(W.prepare(a), W.prepare(b))[0]
        for rs, qs in G.STRANDS:
            exp = G.reference_records(lib, frs, a, b, rs, qs, 11, 23, "c", "q")
            assert D.format_records(frs, a, b, rs, qs, 11, 23, "c", "q") == exp, (k, rs, qs)


def _sam_corpus():
    """SAM text as cut1Gap writes it (dCNS's own records, both strands, hard clip first), plus header, short,
    unclipped and N/S-operator lines; genomes keyed by name."""
    from dcns_gb300 import workloads as W
    from oracle import oracle as O

    orc = O.Oracle()
    rng = np.random.default_rng(4321)
    ref_g, qry_g, lines = {}, {}, ["@HD\tVN:1.6", "@SQ\tSN:chr1\tLN:100", "short"]
    for k in range(3):
        a, b = W.planted_pair(rng, 4000, 3800, 20, 50, 250, 0.88, 0.98, 0.01, 0.2, mask_lo=5, mask_hi=60)
        rname, qname = f"chr{k + 1}", f"ctg{k + 1}"
        ref_g[rname], qry_g[qname] = a, b
        frs = orc.find(W.prepare(a), W.prepare(b))[0]
        for qs in (1, 0):
            sam, _ = D.format_records(frs, a, b, 1, qs, 1, 1, rname, qname)
            lines += sam.splitlines()
    lines += ["ctg1\t0\tchr1\t500\t60\t40M2D10M\t*\t0\t0\tACGT\t*",          # no leading clip: ignored
              "ctg2\t0\tchr2\t700\t60\t12S30M5N20M3I8M\t*\t0\t0\tACGT\t*",   # soft clip, N and I
              "ctg9\t0\tchr1\t100\t60\t7H20M\t*\t0\t0\tACGT\t*",             # query not among the genomes
              "ctg3\t256\tchr3\t900\t60\t3H25M1D9M\t*\t0\t0\tACGT\t*"]       # any non-zero flag
    return "\n".join(lines) + "\n", ref_g, qry_g


def test_sam_to_seeds_matches_reference_reader(tmp_path):
    cli = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libdcns_ref_cli.so")
    if not os.path.exists(cli):
        pytest.skip("reference reader not built on this host")
    import ctypes as C

    sam, ref_g, qry_g = _sam_corpus()
    path = tmp_path / "in.sam"
    path.write_text(sam)
    lib = C.CDLL(cli)
    rn, qn = list(ref_g), list(qry_g)
    arr = lambda xs: (C.c_char_p * len(xs))(*[x.encode() for x in xs])  # noqa: E731
    out = np.zeros((4096, 7), np.int32)
    n = lib.ref_sam_to_seeds(str(path).encode(), len(rn), arr(rn), arr([ref_g[k] for k in rn]), len(qn), arr(qn),
                             arr([qry_g[k] for k in qn]), out.ctypes.data_as(C.POINTER(C.c_int32)), 4096)
    assert n > 20
    exp = {}
    for r in out[:n]:
        key = (int(r[0]), rn[r[1]] if r[1] >= 0 else None, qn[r[2]] if r[2] >= 0 else None)
        exp.setdefault(key, []).append(tuple(int(v) for v in r[3:]))
    got = D.sam_to_seeds(sam, ref_g, qry_g)
    assert got == exp
