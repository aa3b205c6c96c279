"""ORACLE — test infrastructure only (tests/, __graft_entry__.smoke() and bench.py's CPU baseline).

ctypes bindings for two CPU libraries:

* ``liboracle``  — oracle/dcns_oracle.cpp, the scalar restatement of dCNS's pairwise CNS alignment path.  Built on
  every host (here and on the GPU host) by :func:`build`.
* ``libdcns_ref`` — the unmodified reference sources linked with oracle/ref_harness.cpp (oracle/build_ref.sh).
  Only buildable where the reference checkout exists (x86 container); used to pin the restatement and to generate
  the golden fixtures.

Integer parameters travel as ip[13] = match, mismatch, open1, ext1, open2, ext2, window, min_score, step, w, xdrop,
zdrop, bandwidth and doubles as dp[3] = pvalue, lambda, kvalue (defaults: controlLayer4.cpp:28-52 of the reference).
"""
from __future__ import annotations

import ctypes as C
import io
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdcns_ref.so")

DEFAULTS = dict(match=2, mismatch=-3, open1=-4, ext1=-2, open2=-45, ext2=0, window=38, min_score=40, step=8,
                w=10, xdrop=20, zdrop=50, bandwidth=20000, pvalue=0.1, lambda_=0.382291, kvalue=0.006662)

I8P = C.POINTER(C.c_int8)
I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)
U32P = C.POINTER(C.c_uint32)
U64P = C.POINTER(C.c_uint64)
F64P = C.POINTER(C.c_double)


REF_LAZY_SO = os.path.join(HERE, "_ref", "libdcns_ref_lazy.so")
_ref_dir = []


def reference_dir():
    """The reference checkout the parity checker is built from, as oracle/build_ref.sh locates it (the environment
    variable DCNS_REFERENCE overrides the recipe's default); None on hosts without one, which only run built files."""
    if not _ref_dir:
        out = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--where"], capture_output=True, text=True)
        _ref_dir.append(out.stdout.strip() or None)
    return _ref_dir[0]


def build(force: bool = False) -> None:
    """Compile the restatement (always) and the reference harness (where the reference checkout exists)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "dcns_oracle.cpp")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", src, "-o", ORACLE_SO])
    if reference_dir():
        newest = max(os.path.getmtime(os.path.join(HERE, f))
                     for f in ("ref_harness.cpp", "lazy_matrix.cpp", "build_ref.sh"))
        if force or any(not os.path.exists(p) or os.path.getmtime(p) < newest for p in (REF_SO, REF_LAZY_SO)):
            subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")], stdout=subprocess.DEVNULL)


def params(**kw):
    d = dict(DEFAULTS)
    d.update(kw)
    ip = np.array([d["match"], d["mismatch"], d["open1"], d["ext1"], d["open2"], d["ext2"], d["window"],
                   d["min_score"], d["step"], d["w"], d["xdrop"], d["zdrop"], d["bandwidth"]], dtype=np.int32)
    dp = np.array([d["pvalue"], d["lambda_"], d["kvalue"]], dtype=np.float64)
    return d, ip, dp


def _p(a, t):
    return a.ctypes.data_as(t)


def _i8(a):
    a = np.ascontiguousarray(a, dtype=np.int8)
    if a.size == 0:
        a = np.zeros(1, dtype=np.int8)[:0]
    return a


@dataclass
class Fragment:
    """PairedSimilarFragment (model/PairedSimilarFragment.h:14): 1-based coordinates, uint32 score, packed CIGAR."""
    start1: int
    end1: int
    start2: int
    end2: int
    score: int
    cigar: list = field(default_factory=list)
    pvalue: float = 0.0
    evalue: float = 0.0

    def key(self):
        return (self.start1, self.end1, self.start2, self.end2, self.score, tuple(self.cigar))


def _unflatten(n, frag, pe, cig):
    out = []
    for i in range(n):
        r = frag[i]
        out.append(Fragment(int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]),
                            [int(c) for c in cig[int(r[5]):int(r[5]) + int(r[6])]], float(pe[i, 0]), float(pe[i, 1])))
    return out


class _Lib:
    def __init__(self, path):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)


class Oracle(_Lib):
    """The restatement (liboracle.so)."""

    def __init__(self):
        super().__init__(ORACLE_SO)
        L = self.lib
        L.or_sw.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, I32P]
        L.or_xextend.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                 C.c_int, U32P, C.c_int, I32P]
        L.or_semiglobal.argtypes = [I8P, C.c_int32, I8P, C.c_int32, I32P, F64P, C.c_int, U32P, C.c_int, I32P]
        L.or_seeds.argtypes = [I8P, C.c_int32, I8P, C.c_int32, I32P, F64P, C.c_int, I32P, C.c_int, I32P, C.c_int, I32P]
        L.or_find.argtypes = [I8P, C.c_int32, I8P, C.c_int32, I32P, F64P, C.c_int, I64P, F64P, U32P, C.c_int, C.c_int,
                              I32P, I64P]
        L.or_find_batch.argtypes = [C.c_int, C.POINTER(I8P), I32P, C.POINTER(I8P), I32P, I32P, F64P, C.c_int, C.c_int,
                                    I32P, U64P, I64P]
        L.or_sliding.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                 F64P, I32P, C.c_int]
        L.or_xextend_batch.argtypes = [C.c_int, C.POINTER(I8P), I32P, C.POINTER(I8P), I32P] + [C.c_int] * 7 + \
            [I32P, U64P, I64P]
        L.or_find_weighted.argtypes = [C.c_int, I8P, C.c_int32, I8P, C.c_int32, C.POINTER(C.c_int16), I32P, C.c_int32,
                                       I32P, F64P, I64P, F64P, U32P, C.c_int, C.c_int, I32P, I64P]
        L.or_find_seeded_2gap.argtypes = [I8P, C.c_int32, I8P, C.c_int32, I32P, C.c_int32, C.c_int32, I32P, F64P, I64P,
                                          F64P, U32P, C.c_int, C.c_int, I32P, I64P]
        L.or_find_xseeds_2gap.argtypes = [I8P, C.c_int32, I8P, C.c_int32, I32P, C.c_int32, I32P, F64P, I64P, F64P,
                                          U32P, C.c_int, C.c_int, I32P, I64P]

    def sw(self, ref, read, open=-4, ext=-2, match=2, mismatch=-3, mode=0):
        """mode 0: the reference's own dispatch; 1: striped (AVX2) semantics; 2: scalar semantics."""
        ref, read = _i8(ref), _i8(read)
        out = np.zeros(3, np.int32)
        self.lib.or_sw(_p(ref, I8P), len(ref), _p(read, I8P), len(read), open, ext, match, mismatch, mode,
                       _p(out, I32P))
        return tuple(int(x) for x in out)

    def xextend(self, s1, s2, open=-4, ext=-2, match=2, mismatch=-3, xdrop=20, w=10, cigar=False):
        s1, s2 = _i8(s1), _i8(s2)
        cap = len(s1) + len(s2) + 8
        cg = np.zeros(cap, np.uint32)
        out = np.zeros(7, np.int32)
        rc = self.lib.or_xextend(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), open, ext, match, mismatch, xdrop, w,
                                 int(cigar), _p(cg, U32P), cap, _p(out, I32P))
        assert rc == 0
        return dict(score=int(out[0]), end1=int(out[1]), end2=int(out[2]), iii=int(out[3]), jjj=int(out[4]),
                    cigar=[int(c) for c in cg[:out[5]]], cells=int(out[6]))

    def semiglobal(self, s1, s2, cigar=False, **kw):
        _, ip, dp = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        cap = len(s1) + len(s2) + 8
        cg = np.zeros(cap, np.uint32)
        out = np.zeros(4, np.int32)
        rc = self.lib.or_semiglobal(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), _p(ip, I32P), _p(dp, F64P),
                                    int(cigar), _p(cg, U32P), cap, _p(out, I32P))
        assert rc == 0
        return dict(score=int(out[0]), end1=int(out[1]), end2=int(out[2]), cigar=[int(c) for c in cg[:out[3]]])

    def seeds(self, s1, s2, one_gap=True, **kw):
        _, ip, dp = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        cap = 1 << 16
        raw = np.zeros((cap, 4), np.int32)
        lk = np.zeros((cap, 4), np.int32)
        nl = np.zeros(1, np.int32)
        n = self.lib.or_seeds(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), _p(ip, I32P), _p(dp, F64P), int(one_gap),
                              _p(raw, I32P), cap, _p(lk, I32P), cap, _p(nl, I32P))
        return [tuple(int(v) for v in r) for r in raw[:n]], [tuple(int(v) for v in r) for r in lk[:nl[0]]]

    def find(self, s1, s2, two_gap=False, **kw):
        _, ip, dp = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        cells = np.zeros(4, np.int64)
        n = self.lib.or_find(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), _p(ip, I32P), _p(dp, F64P), int(two_gap),
                             _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap, ccap, _p(nc, I32P), _p(cells, I64P))
        assert n >= 0, "fragment buffer too small"
        return _unflatten(n, frag, pe, cg), dict(zip(("scan", "scan_rev", "xdrop", "semiglobal"), map(int, cells)))

    def find_weighted(self, s1, s2, weights, cats, pieces=2, **kw):
        """The weighted drivers: weights = category id per base of s1, cats = [(match, mismatch, open1, ext1, open2,
        ext2, zdrop), ...]; pieces 1 = the 1-gap weighted driver, 2 = the 2-gap one."""
        _, ip, dp = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        wt = np.ascontiguousarray(weights, np.int16)
        ct = np.ascontiguousarray(cats, np.int32).reshape(-1, 7)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        cells = np.zeros(4, np.int64)
        n = self.lib.or_find_weighted(pieces, _p(s1, I8P), len(s1), _p(s2, I8P), len(s2),
                                      wt.ctypes.data_as(C.POINTER(C.c_int16)), _p(ct, I32P), len(ct), _p(ip, I32P),
                                      _p(dp, F64P), _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap, ccap,
                                      _p(nc, I32P), _p(cells, I64P))
        assert n >= 0, "fragment buffer too small"
        return _unflatten(n, frag, pe, cg)

    def find_seeded(self, s1, s2, seeds, max_align=20000, with_cells=False, **kw):
        """The seeded 2-piece overload (cut2Gaps2): seeds = [(start1, end1, start2, end2)] 0-based, in order.  With
        with_cells, also the algorithmic cells it evaluated ({"scan", "scan_rev", "xdrop", "semiglobal"})."""
        _, ip, dp = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        sd = np.asarray(seeds, np.int32).reshape(-1, 4)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        cells = np.zeros(4, np.int64)
        n = self.lib.or_find_seeded_2gap(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), _p(sd, I32P), len(sd), max_align,
                                         _p(ip, I32P), _p(dp, F64P), _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap,
                                         ccap, _p(nc, I32P), _p(cells, I64P))
        assert n >= 0, "fragment buffer too small"
        out = _unflatten(n, frag, pe, cg)
        if with_cells:
            return out, dict(zip(("scan", "scan_rev", "xdrop", "semiglobal"), map(int, cells)))
        return out

    def find_xseeds(self, s1, s2, seeds, **kw):
        """The x-seed overload without maximumAlignLength (findSimilar...4.cpp:532): seeds = [(start1, end1, start2,
        end2)] 0-based, in order."""
        _, ip, dp = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        sd = np.asarray(seeds, np.int32).reshape(-1, 4)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        cells = np.zeros(4, np.int64)
        n = self.lib.or_find_xseeds_2gap(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), _p(sd, I32P), len(sd),
                                         _p(ip, I32P), _p(dp, F64P), _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap,
                                         ccap, _p(nc, I32P), _p(cells, I64P))
        assert n >= 0, "fragment buffer too small"
        return _unflatten(n, frag, pe, cg)

    def find_batch(self, pairs, two_gap=False, threads=1, **kw):
        """pairs: list of (seq1 codes, seq2 codes).  Returns (n_fragments per pair, checksum, cells)."""
        _, ip, dp = params(**kw)
        keep = [(_i8(a), _i8(b)) for a, b in pairs]
        n = len(keep)
        p1 = (I8P * n)(*[_p(a, I8P) for a, _ in keep])
        p2 = (I8P * n)(*[_p(b, I8P) for _, b in keep])
        n1 = np.array([len(a) for a, _ in keep], np.int32)
        n2 = np.array([len(b) for _, b in keep], np.int32)
        nf = np.zeros(n, np.int32)
        ck = np.zeros(1, np.uint64)
        cells = np.zeros(4, np.int64)
        self.lib.or_find_batch(n, p1, _p(n1, I32P), p2, _p(n2, I32P), _p(ip, I32P), _p(dp, F64P), int(two_gap),
                               int(threads), _p(nf, I32P), _p(ck, U64P), _p(cells, I64P))
        return nf, int(ck[0]), dict(zip(("scan", "scan_rev", "xdrop", "semiglobal"), map(int, cells)))

    def xextend_batch(self, tasks, threads=1, open=-4, ext=-2, match=2, mismatch=-3, xdrop=20, w=10):
        """x_extend_seed's two passes (forward, then with traceback) per (seq1, seq2) task on `threads` threads.
        Returns (traceback-pass scores, checksum, algorithmic cells of both passes)."""
        keep = [(_i8(a), _i8(b)) for a, b in tasks]
        n = len(keep)
        p1 = (I8P * max(n, 1))(*[_p(a, I8P) for a, _ in keep])
        p2 = (I8P * max(n, 1))(*[_p(b, I8P) for _, b in keep])
        n1 = np.array([len(a) for a, _ in keep] or [0], np.int32)
        n2 = np.array([len(b) for _, b in keep] or [0], np.int32)
        out = np.zeros(max(n, 1), np.int32)
        ck = np.zeros(1, np.uint64)
        cells = np.zeros(1, np.int64)
        self.lib.or_xextend_batch(n, p1, _p(n1, I32P), p2, _p(n2, I32P), open, ext, match, mismatch, xdrop, w,
                                  int(threads), _p(out, I32P), _p(ck, U64P), _p(cells, I64P))
        return out[:n], int(ck[0]), int(cells[0])

    def sliding(self, ref, other, window=38, step=8, open=-4, ext=-2, match=2, mismatch=-3):
        ref, other = _i8(ref), _i8(other)
        cap = len(ref) // max(step, 1) + 2
        sc = np.zeros(cap, np.float64)
        mx = np.zeros(cap, np.int32)
        n = self.lib.or_sliding(_p(ref, I8P), len(ref), _p(other, I8P), len(other), window, step, open, ext, match,
                                mismatch, _p(sc, F64P), _p(mx, I32P), cap)
        return sc[:n].copy(), mx[:n].copy()


class Reference(_Lib):
    """The unmodified reference behind oracle/ref_harness.cpp (libdcns_ref.so).  lazy=True loads the same code with
    oracle/lazy_matrix.cpp in place of its dense traceback matrix (libdcns_ref_lazy.so), for pairs whose dense matrix
    would not fit in memory."""

    def __init__(self, lazy: bool = False):
        super().__init__(REF_LAZY_SO if lazy else REF_SO)
        L = self.lib
        L.ref_sw.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, I32P]
        L.ref_sw_scalar.argtypes = L.ref_sw.argtypes
        L.ref_find_weighted.argtypes = [C.c_int, I8P, C.c_int32, I8P, C.c_int32, C.POINTER(C.c_int16), I32P,
                                        C.c_int32, C.c_char_p] + [C.c_int] * 7 + [C.c_double] * 3 + \
            [C.c_int] * 4 + [I64P, F64P, U32P, C.c_int, C.c_int, I32P]
        L.ref_find_seeded_2gap.argtypes = [I8P, C.c_int32, I8P, C.c_int32, I32P, C.c_int32, C.c_int32] + \
            [C.c_int] * 6 + [C.c_double] * 3 + [C.c_int, C.c_int, I64P, F64P, U32P, C.c_int, C.c_int, I32P]
        L.ref_find_xseeds_2gap.argtypes = [I8P, C.c_int32, I8P, C.c_int32, I32P, C.c_int32] + \
            [C.c_int] * 6 + [C.c_double] * 3 + [C.c_int, C.c_int, I64P, F64P, U32P, C.c_int, C.c_int, I32P]
        L.ref_xextend.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_int, I32P]
        L.ref_xextend_cigar.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, U32P, C.c_int, I32P]
        L.ref_semiglobal.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.c_int, C.c_int, C.c_int, C.c_int, U32P, C.c_int, I32P]
        L.ref_seeds_1gap.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.c_int, C.c_int, I32P, C.c_int, I32P, C.c_int, I32P]
        L.ref_find_1gap.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, I64P, F64P,
                                    U32P, C.c_int, C.c_int, I32P]
        L.ref_find_2gap.argtypes = [I8P, C.c_int32, I8P, C.c_int32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                    C.c_int, C.c_int, C.c_int, I64P, F64P, U32P, C.c_int, C.c_int, I32P]
        L.ref_sliding.argtypes = [C.POINTER(I8P), I32P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_char_p]

    def sw(self, ref, read, open=-4, ext=-2, match=2, mismatch=-3, scalar=False):
        ref, read = _i8(ref), _i8(read)
        out = np.zeros(3, np.int32)
        f = self.lib.ref_sw_scalar if scalar else self.lib.ref_sw
        f(_p(ref, I8P), len(ref), _p(read, I8P), len(read), open, ext, match, mismatch, _p(out, I32P))
        return tuple(int(x) for x in out)

    def xextend(self, s1, s2, open=-4, ext=-2, match=2, mismatch=-3, xdrop=20, w=10, cigar=False):
        s1, s2 = _i8(s1), _i8(s2)
        if not cigar:
            out = np.zeros(3, np.int32)
            self.lib.ref_xextend(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), open, ext, match, mismatch, xdrop, w,
                                 _p(out, I32P))
            return dict(score=int(out[0]), end1=int(out[1]), end2=int(out[2]), iii=0, jjj=0, cigar=[])
        cap = len(s1) + len(s2) + 8
        cg = np.zeros(cap, np.uint32)
        out = np.zeros(6, np.int32)
        rc = self.lib.ref_xextend_cigar(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), open, ext, match, mismatch, xdrop,
                                        w, _p(cg, U32P), cap, _p(out, I32P))
        assert rc == 0
        return dict(score=int(out[0]), end1=int(out[1]), end2=int(out[2]), iii=int(out[3]), jjj=int(out[4]),
                    cigar=[int(c) for c in cg[:out[5]]])

    def semiglobal(self, s1, s2, cigar=False, **kw):
        d, _, _ = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        cap = len(s1) + len(s2) + 8
        cg = np.zeros(cap, np.uint32)
        out = np.zeros(4, np.int32)
        rc = self.lib.ref_semiglobal(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), d["open1"], d["ext1"], d["open2"],
                                     d["ext2"], d["match"], d["mismatch"], int(cigar), d["zdrop"], d["bandwidth"],
                                     _p(cg, U32P), cap, _p(out, I32P))
        assert rc == 0
        return dict(score=int(out[0]), end1=int(out[1]), end2=int(out[2]), cigar=[int(c) for c in cg[:out[3]]])

    def seeds(self, s1, s2, **kw):
        d, _, _ = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        cap = 1 << 16
        raw = np.zeros((cap, 4), np.int32)
        lk = np.zeros((cap, 4), np.int32)
        nl = np.zeros(1, np.int32)
        n = self.lib.ref_seeds_1gap(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), d["window"], d["min_score"],
                                    d["open1"], d["ext1"], d["match"], d["mismatch"], d["step"], _p(raw, I32P), cap,
                                    _p(lk, I32P), cap, _p(nl, I32P))
        return [tuple(int(v) for v in r) for r in raw[:n]], [tuple(int(v) for v in r) for r in lk[:nl[0]]]

    def find(self, s1, s2, two_gap=False, **kw):
        d, _, _ = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        if two_gap:
            n = self.lib.ref_find_2gap(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), d["window"], d["min_score"],
                                       d["open1"], d["ext1"], d["open2"], d["ext2"], d["match"], d["mismatch"],
                                       d["step"], d["pvalue"], d["lambda_"], d["kvalue"], d["zdrop"], d["bandwidth"],
                                       d["w"], d["xdrop"], _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap, ccap,
                                       _p(nc, I32P))
        else:
            n = self.lib.ref_find_1gap(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), d["window"], d["min_score"],
                                       d["open1"], d["ext1"], d["match"], d["mismatch"], d["step"], d["pvalue"],
                                       d["lambda_"], d["kvalue"], d["w"], d["xdrop"], _p(frag, I64P), _p(pe, F64P),
                                       _p(cg, U32P), fcap, ccap, _p(nc, I32P))
        assert n >= 0, "fragment buffer too small"
        return _unflatten(n, frag, pe, cg)

    def find_weighted(self, s1, s2, weights, cats, pieces=2, **kw):
        import tempfile
        d, _, _ = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        wt = np.ascontiguousarray(weights, np.int16)
        ct = np.ascontiguousarray(cats, np.int32).reshape(-1, 7)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        with tempfile.TemporaryDirectory() as sd:
            n = self.lib.ref_find_weighted(pieces, _p(s1, I8P), len(s1), _p(s2, I8P), len(s2),
                                           wt.ctypes.data_as(C.POINTER(C.c_int16)), _p(ct, I32P), len(ct),
                                           sd.encode(), d["window"], d["min_score"], d["open1"], d["ext1"],
                                           d["match"], d["mismatch"], d["step"], d["pvalue"], d["lambda_"],
                                           d["kvalue"], d["zdrop"], d["bandwidth"], d["w"], d["xdrop"],
                                           _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap, ccap, _p(nc, I32P))
        assert n >= 0, "fragment buffer too small"
        return _unflatten(n, frag, pe, cg)

    def find_seeded(self, s1, s2, seeds, max_align=20000, **kw):
        d, _, _ = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        sd = np.asarray(seeds, np.int32).reshape(-1, 4)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        n = self.lib.ref_find_seeded_2gap(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), _p(sd, I32P), len(sd),
                                          max_align, d["open1"], d["ext1"], d["open2"], d["ext2"], d["match"],
                                          d["mismatch"], d["pvalue"], d["lambda_"], d["kvalue"], d["zdrop"],
                                          d["bandwidth"], _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap, ccap,
                                          _p(nc, I32P))
        assert n >= 0, "fragment buffer too small"
        return _unflatten(n, frag, pe, cg)

    def find_xseeds(self, s1, s2, seeds, **kw):
        d, _, _ = params(**kw)
        s1, s2 = _i8(s1), _i8(s2)
        sd = np.asarray(seeds, np.int32).reshape(-1, 4)
        fcap, ccap = 4096, 1 << 20
        frag = np.zeros((fcap, 8), np.int64)
        pe = np.zeros((fcap, 2), np.float64)
        cg = np.zeros(ccap, np.uint32)
        nc = np.zeros(1, np.int32)
        n = self.lib.ref_find_xseeds_2gap(_p(s1, I8P), len(s1), _p(s2, I8P), len(s2), _p(sd, I32P), len(sd),
                                          d["open1"], d["ext1"], d["open2"], d["ext2"], d["match"], d["mismatch"],
                                          d["pvalue"], d["lambda_"], d["kvalue"], d["zdrop"], d["bandwidth"],
                                          _p(frag, I64P), _p(pe, F64P), _p(cg, U32P), fcap, ccap, _p(nc, I32P))
        assert n >= 0, "fragment buffer too small"
        return _unflatten(n, frag, pe, cg)

    def sliding(self, seqs, window=38, step=8, open=-4, ext=-2, match=2, mismatch=-3, path=None):
        """Runs slidingWindowAlignment and parses its "j name score" lines -> list of (j, seq_index, score)."""
        import tempfile
        keep = [_i8(s) for s in seqs]
        ptrs = (I8P * len(keep))(*[_p(s, I8P) for s in keep])
        lens = np.array([len(s) for s in keep], np.int32)
        with tempfile.TemporaryDirectory() as td:
            out = path or os.path.join(td, "slide.txt")
            self.lib.ref_sliding(ptrs, _p(lens, I32P), len(keep), window, step, open, ext, match, mismatch,
                                 out.encode())
            rows = []
            with io.open(out) as fh:
                for line in fh:
                    j, name, sc = line.split()
                    rows.append((int(j), int(name[1:]), sc))
        return rows
