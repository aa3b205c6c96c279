"""dcns_gb300 — GB300-native pairwise CNS alignment (dCNS's seed scan, x-drop extension and 2-piece semi-global DP).

The engine is a C-ABI shared library (``include/dcns_gb300.h``, built from ``dcns_gb300/csrc`` for sm_103a) driven
through ctypes.  This module builds it in-tree, loads it, and mirrors the reference's entry points:

* :meth:`Engine.findSimilarFragmentsForPairedSequence` — the 1-gap / 2-gap overloads
  (impl/findSimilarFragmentsForPairedSequence.h:26-42 of the reference) for one pair,
* :meth:`Engine.align_pairs` — the batched form (many independent pairs in one call),
* :meth:`Engine.SmithWaterman`, :meth:`Engine.SemiGlobal_xextend`, :meth:`Engine.SemiGlobal` and
  :meth:`Engine.slidingWindowAlignment` — the kernel-level functions (impl/sequenceAlignment.h:18-88,
  impl/slidingWindowAlignment.h:21-24).

There is no CPU fallback: :func:`load` raises when the library is missing or no CUDA device is usable.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from collections.abc import Sequence
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libdcnsgpu.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

MODE_ONE_GAP = 1
MODE_TWO_GAP = 2

ERRORS = {-1: "invalid argument", -2: "out of memory", -3: "device error", -4: "timeout", -5: "not found",
          -6: "busy"}


class DcnsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "dcns_gb300.h")]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA/C++ source for sm_103a into dcns_gb300/_lib/libdcnsgpu.so (in-tree, parallel).  Processes
    that call this at once (one per rank) take turns on a lock file; the later ones find the library current."""
    import fcntl

    os.makedirs(LIBDIR, exist_ok=True)
    with open(os.path.join(LIBDIR, ".build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build_locked(force, verbose)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(force: bool, verbose: bool) -> str:
    srcs = _sources()
    newest = max(os.path.getmtime(p) for p in srcs + _headers())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    nvcc = os.environ.get("NVCC", "nvcc")
    common = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC] + ARCH

    def compile_one(src):
        obj = os.path.join(LIBDIR, os.path.basename(src) + ".o")
        cmd = [nvcc] + common + ["-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc, "-shared"] + ARCH + objs + ["-o", tmp, "-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


# ------------------------------------------------------------------ ctypes mirror of include/dcns_gb300.h
class Params(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("match", "mismatch", "open1", "ext1", "open2", "ext2", "window",
                                         "min_score", "step", "w", "xdrop", "zdrop", "bandwidth",
                                         "max_align_len")] + [("pvalue", C.c_double), ("lambda_", C.c_double),
                                                              ("kvalue", C.c_double)]


class Pair(C.Structure):
    _fields_ = [("seq1", C.POINTER(C.c_int8)), ("len1", C.c_int32), ("seq2", C.POINTER(C.c_int8)),
                ("len2", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("cells_scan", "cells_scan_reverse", "cells_xdrop", "cells_semiglobal",
                                         "tasks_scan", "tasks_scan_speculative", "seeds", "xdrop_passes",
                                         "semiglobal_dps")] + \
               [(n, C.c_double) for n in ("ms_upload", "ms_scan", "ms_replay", "ms_xdrop", "ms_semiglobal",
                                          "ms_download", "ms_total", "ms_scan_kernel", "ms_scan_prep",
                                          "ms_scan_xfer", "ms_link")] + \
               [("scan_launches", C.c_int32), ("kernel_launches", C.c_int32), ("scan_rounds", C.c_int32),
                ("xdrop_rounds", C.c_int32), ("ms_xdrop_kernel", C.c_double), ("bytes_h2d", C.c_int64),
                ("ms_xdrop_tb_kernel", C.c_double), ("ms_sg_kernel", C.c_double), ("ms_sg_tb_kernel", C.c_double),
                ("bytes_codes_xdrop", C.c_int64), ("bytes_codes_sg", C.c_int64), ("bytes_device", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServingStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "cancelled", "batches", "max_batch",
                                         "nomem_splits", "solo_retries", "queued", "pending")] + \
               [("workers", C.c_int32), ("pad", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class Tuning(C.Structure):
    _fields_ = [("lanes", C.c_int32), ("bins", C.c_int32), ("bin_ratio", C.c_double),
                ("scan_tiles_per_thread", C.c_int32), ("sg_warps", C.c_int32), ("sg_flow", C.c_int32), ("sg_flow_blocks", C.c_int32),
                ("bins_by_size", C.c_int32),
                ("n_bins_tuned", C.c_int32),
                ("xdrop_warp_from", C.c_int32 * 16), ("xdrop_wave_max_w", C.c_int32 * 16), ("xdrop_flat", C.c_int32 * 16),
                ("xdrop_handoff", C.c_int32 * 16), ("xdrop_resume_lanes", C.c_int32 * 16),
                ("xdrop_group_from", C.c_int32 * 16), ("scan_tiles", C.c_int32 * 16)]

    def as_dict(self):
        n = max(self.n_bins_tuned, 1)
        return {"lanes": self.lanes, "bins": self.bins, "bin_ratio": self.bin_ratio,
                "scan_tiles_per_thread": self.scan_tiles_per_thread, "sg_warps": self.sg_warps,
                "sg_flow": bool(self.sg_flow), "sg_flow_blocks": self.sg_flow_blocks,
                "bins_by_size": bool(self.bins_by_size),
                "xdrop_per_bin": [{"warp_from": self.xdrop_warp_from[b], "wave_max_w": self.xdrop_wave_max_w[b],
                                   "row_interleaved": bool(self.xdrop_flat[b]),
                                   "handoff_rows": self.xdrop_handoff[b],
                                   "handoff_lanes": self.xdrop_resume_lanes[b],
                                   "groups_from_band": self.xdrop_group_from[b],
                                   "scan_tiles": self.scan_tiles[b]} for b in range(n)]}


class Results(C.Structure):
    _fields_ = [("n_pairs", C.c_int64), ("n_fragments", C.c_int64), ("n_cigar", C.c_int64),
                ("pair_offset", C.POINTER(C.c_int64)), ("frag", C.POINTER(C.c_int64)),
                ("pvalue", C.POINTER(C.c_double)), ("evalue", C.POINTER(C.c_double)),
                ("cigar", C.POINTER(C.c_uint32)), ("stats", Stats)]


@dataclass
class Fragment:
    """PairedSimilarFragment (model/PairedSimilarFragment.h:14 of the reference): 1-based coordinates, uint32 score,
    CIGAR words (length << 4 | op; op 0=M, 1=I, 2=D), FP64 p- and e-value."""
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


_I8P = C.POINTER(C.c_int8)
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_U32P = C.POINTER(C.c_uint32)
_F64P = C.POINTER(C.c_double)
P16 = C.POINTER(C.c_int16)


def _bind(lib):
    P = C.POINTER
    lib.dcns_params_default.argtypes = [P(Params)]
    lib.dcns_ctx_create.argtypes = [C.c_int, C.c_size_t, P(C.c_void_p)]
    lib.dcns_ctx_destroy.argtypes = [C.c_void_p]
    lib.dcns_last_error.argtypes = [C.c_void_p]
    lib.dcns_last_error.restype = C.c_char_p
    lib.dcns_ctx_stream.argtypes = [C.c_void_p]
    lib.dcns_ctx_stream.restype = C.c_void_p
    lib.dcns_align_pairs.argtypes = [C.c_void_p, P(Pair), C.c_int64, P(Params), C.c_int, P(P(Results))]
    lib.dcns_results_free.argtypes = [P(Results)]
    lib.dcns_last_stats.argtypes = [C.c_void_p, P(Stats)]
    lib.dcns_ctx_set_lanes.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.dcns_align_weighted.argtypes = [C.c_void_p, P(Pair), C.c_int64, P(C.c_int16), _I32P, C.c_int32, C.c_int,
                                        P(Params), P(P(Results))]
    lib.dcns_align_seeded.argtypes = [C.c_void_p, P(Pair), C.c_int64, _I32P, _I64P, P(Params), P(P(Results))]
    lib.dcns_align_xseeds.argtypes = lib.dcns_align_seeded.argtypes
    lib.dcns_format_records.argtypes = [C.c_int64, _I64P, _U32P, _F64P, C.c_char_p, C.c_int64, C.c_char_p,
                                        C.c_int64, C.c_int, C.c_int, C.c_int32, C.c_int32, C.c_char_p, C.c_char_p,
                                        P(C.c_void_p), P(C.c_int64), P(C.c_void_p), P(C.c_int64)]
    lib.dcns_free_text.argtypes = [C.c_void_p]
    lib.dcns_sam_to_seeds.argtypes = [C.c_char_p, C.c_int64, C.c_int, P(C.c_char_p), P(C.c_char_p), _I64P, C.c_int,
                                      P(C.c_char_p), P(C.c_char_p), _I64P, P(_I32P), P(C.c_int64)]
    lib.dcns_free_seeds.argtypes = [_I32P]
    lib.dcns_autotune.argtypes = [C.c_void_p, C.c_void_p, P(Params), C.c_int, P(C.c_int), P(C.c_int),
                                  P(C.c_double)]
    lib.dcns_smith_waterman_batch.argtypes = [C.c_void_p, P(Pair), C.c_int64, P(Params), _I32P]
    lib.dcns_xextend_batch.argtypes = [C.c_void_p, P(Pair), C.c_int64, P(Params), C.c_int, _I32P, _U32P, C.c_int64,
                                       _I64P]
    lib.dcns_semiglobal_batch.argtypes = lib.dcns_xextend_batch.argtypes
    lib.dcns_sliding_window.argtypes = [C.c_void_p, P(_I8P), _I32P, C.c_int32, P(Params), _F64P, _I32P]
    lib.dcns_batch_upload.argtypes = [C.c_void_p, P(Pair), C.c_int64, P(C.c_void_p)]
    lib.dcns_align_batch.argtypes = [C.c_void_p, C.c_void_p, P(Params), C.c_int, P(P(Results))]
    lib.dcns_batch_free.argtypes = [C.c_void_p, C.c_void_p]
    lib.dcns_measure_scan_roofline.argtypes = [C.c_void_p, P(C.c_double)]
    lib.dcns_serve_start.argtypes = [C.c_void_p, P(Params), C.c_int, C.c_int]
    lib.dcns_submit.argtypes = [C.c_void_p, P(Pair), P(C.c_uint64)]
    lib.dcns_poll.argtypes = [C.c_void_p, C.c_uint64, P(P(Results))]
    lib.dcns_serve_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_int64, P(P(Results))]
    lib.dcns_serve_stop.argtypes = [C.c_void_p]
    lib.dcns_cancel.argtypes = [C.c_void_p, C.c_uint64]
    lib.dcns_get_tuning.argtypes = [C.c_void_p, P(Tuning)]
    lib.dcns_serve_set_shape.argtypes = [C.c_void_p, C.c_int, C.c_int64, C.c_int64]
    lib.dcns_serve_stats.argtypes = [C.c_void_p, P(ServingStats)]
    return lib


_lib = None
_lock = threading.Lock()


def library():
    """The loaded C-ABI library (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB):
                raise RuntimeError(f"{LIB} is missing: call dcns_gb300.build() (no CPU fallback exists)")
            _lib = _bind(C.CDLL(LIB))
    return _lib


def format_records(fragments, ref_text: str, qry_text: str, ref_strand: int = 1, qry_strand: int = 1,
                   ref_start: int = 1, qry_start: int = 1, ref_chr: str = "ref", qry_chr: str = "query"):
    """SAM and "o" text of one pair as cut1Gap writes them (outputMasking, controlLayer4.cpp:835-1358): `fragments` of
    that pair (from align_pairs), the region texts still holding their lower-case 'n' runs, strands (1 +, 0 -),
    1-based region starts and names.  Host only; returns (sam_text, o_text)."""
    frs = list(fragments)
    n = len(frs)
    frag = np.zeros((max(n, 1), 7), np.int64)
    cig, pv = [], np.zeros(max(n, 1), np.float64)
    for k, f in enumerate(frs):
        frag[k, :5] = (f.start1, f.end1, f.start2, f.end2, f.score)
        frag[k, 5], frag[k, 6] = len(cig), len(f.cigar)
        cig.extend(int(c) for c in f.cigar)
        pv[k] = f.pvalue
    cg = np.asarray(cig if cig else [0], np.uint32)
    t1, t2 = ref_text.encode(), qry_text.encode()
    sam, o, ls, lo = C.c_void_p(), C.c_void_p(), C.c_int64(), C.c_int64()
    lib = library()
    rc = lib.dcns_format_records(n, frag.ctypes.data_as(_I64P), cg.ctypes.data_as(_U32P), pv.ctypes.data_as(_F64P),
                                 t1, len(t1), t2, len(t2), int(ref_strand), int(qry_strand), int(ref_start),
                                 int(qry_start), ref_chr.encode(), qry_chr.encode(), C.byref(sam), C.byref(ls),
                                 C.byref(o), C.byref(lo))
    if rc != 0:
        raise DcnsError(rc, "format_records failed")
    try:
        return C.string_at(sam, ls.value).decode(), C.string_at(o, lo.value).decode()
    finally:
        lib.dcns_free_text(sam)
        lib.dcns_free_text(o)


def sam_to_seeds(sam_text: str, ref_genome: dict, query_genome: dict):
    """cut2Gaps2's x-seeds from SAM text (samFileToSeeds): {(strand, ref name, query name): [(start1, end1, start2,
    end2), ...]} in line order, strand 0 for flag 0 and 1 otherwise; genomes map names to texts with 'n' runs."""
    rn, qn = list(ref_genome), list(query_genome)
    rb = [ref_genome[k].encode() for k in rn]
    qb = [query_genome[k].encode() for k in qn]
    arr = lambda xs: (C.c_char_p * max(1, len(xs)))(*xs)  # noqa: E731
    rl = np.array([len(x) for x in rb] or [0], np.int64)
    ql = np.array([len(x) for x in qb] or [0], np.int64)
    sam = sam_text.encode()
    out, n = _I32P(), C.c_int64()
    lib = library()
    rc = lib.dcns_sam_to_seeds(sam, len(sam), len(rn), arr([k.encode() for k in rn]), arr(rb), rl.ctypes.data_as(_I64P),
                               len(qn), arr([k.encode() for k in qn]), arr(qb), ql.ctypes.data_as(_I64P),
                               C.byref(out), C.byref(n))
    if rc != 0:
        raise DcnsError(rc, "sam_to_seeds failed")
    try:
        recs = np.ctypeslib.as_array(out, shape=(max(1, n.value) * 7,))[:n.value * 7].reshape(-1, 7).copy()
    finally:
        lib.dcns_free_seeds(out)
    seeds = {}
    for r in recs:
        key = (int(r[2]), rn[r[0]] if r[0] >= 0 else None, qn[r[1]] if r[1] >= 0 else None)
        seeds.setdefault(key, []).append(tuple(int(v) for v in r[3:]))
    return seeds


def params(**kw) -> Params:
    p = Params()
    library().dcns_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, "lambda_" if k == "lambda" else k, v)
    return p


def _codes(a):
    a = np.ascontiguousarray(a, dtype=np.int8)
    return a


_PAIR_DT = np.dtype({"names": ["seq1", "len1", "seq2", "len2"], "formats": ["<u8", "<i4", "<u8", "<i4"],
                     "offsets": [Pair.seq1.offset, Pair.len1.offset, Pair.seq2.offset, Pair.len2.offset],
                     "itemsize": C.sizeof(Pair)})


def _pairs(pairs):
    """dcns_pair array pointing at the callers' sequences (contiguous int8 views; copies only where a sequence is not
    already one).  Returns (array, keep-alive object whose len() is the number of pairs)."""
    n = len(pairs)
    if n == 0:
        return (Pair * 1)(), _Keep(0, ())
    seqs = [_codes(x).reshape(-1) for ab in pairs for x in ab]
    if len(seqs) != 2 * n:
        raise ValueError("every pair must hold exactly two sequences")
    ptr = np.fromiter((x.ctypes.data for x in seqs), np.uint64, 2 * n)
    lens = np.fromiter((x.shape[0] for x in seqs), np.int64, 2 * n)
    sa = np.zeros(n, _PAIR_DT)
    sa["seq1"], sa["seq2"] = ptr[0::2], ptr[1::2]
    sa["len1"], sa["len2"] = lens[0::2], lens[1::2]
    arr = (Pair * n).from_buffer(sa)
    return arr, _Keep(n, (seqs, sa))


class _Keep(tuple):
    """Keeps the concatenated sequences alive; len() is the number of pairs."""

    def __new__(cls, n, objs):
        t = super().__new__(cls, objs)
        t.n = n
        return t

    def __len__(self):
        return self.n


class FragmentList:
    """The fragments of one pair, materialised lazily from the flat result arrays."""

    __slots__ = ("_frag", "_pv", "_ev", "_cg", "_lo", "_hi")

    def __init__(self, frag, pv, ev, cg, lo, hi):
        self._frag, self._pv, self._ev, self._cg, self._lo, self._hi = frag, pv, ev, cg, lo, hi

    def __len__(self):
        return self._hi - self._lo

    def __getitem__(self, k):
        if isinstance(k, slice):
            return [self[i] for i in range(*k.indices(len(self)))]
        if k < 0:
            k += len(self)
        if not 0 <= k < len(self):
            raise IndexError(k)
        i = self._lo + k
        r = self._frag[i]
        return Fragment(int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]),
                        self._cg[int(r[5]):int(r[5]) + int(r[6])].tolist(), float(self._pv[i]), float(self._ev[i]))

    def __iter__(self):
        return (self[k] for k in range(len(self)))

    def __eq__(self, other):
        return list(self) == list(other)

    def __repr__(self):
        return f"FragmentList({list(self)!r})"


def _unpack(res):
    """Copies the flat C results into numpy arrays; per-pair views build Fragment objects only when accessed."""
    R = res.contents
    n = int(R.n_pairs)
    if n == 0:
        return []
    off = np.ctypeslib.as_array(R.pair_offset, shape=(n + 1,)).copy()
    nf = int(R.n_fragments)
    nc = int(R.n_cigar)
    frag = np.ctypeslib.as_array(R.frag, shape=(nf * 7,)).reshape(nf, 7).copy() if nf else np.zeros((0, 7), np.int64)
    pv = np.ctypeslib.as_array(R.pvalue, shape=(nf,)).copy() if nf else np.zeros(0)
    ev = np.ctypeslib.as_array(R.evalue, shape=(nf,)).copy() if nf else np.zeros(0)
    cg = np.ctypeslib.as_array(R.cigar, shape=(nc,)).copy() if nc else np.zeros(0, np.uint32)
    return BatchResults(off, frag, pv, ev, cg)


class BatchResults(Sequence):
    """Per-pair fragment lists of one call (a read-only sequence indexed like the input pairs); each pair's
    FragmentList is made when it is accessed.  The flat arrays are public: frag (rows of start1, end1, start2, end2,
    score, cigar offset, cigar length), pvalue, evalue, cigar, pair_offset."""

    __slots__ = ("pair_offset", "frag", "pvalue", "evalue", "cigar")

    def __init__(self, off, frag, pv, ev, cg):
        self.pair_offset, self.frag, self.pvalue, self.evalue, self.cigar = off, frag, pv, ev, cg

    def __len__(self):
        return len(self.pair_offset) - 1

    def __getitem__(self, k):
        if isinstance(k, slice):
            return [self[i] for i in range(*k.indices(len(self)))]
        n = len(self)
        if k < 0:
            k += n
        if not 0 <= k < n:
            raise IndexError(k)
        return FragmentList(self.frag, self.pvalue, self.evalue, self.cigar, int(self.pair_offset[k]),
                            int(self.pair_offset[k + 1]))

    def n_fragments(self) -> int:
        return int(self.pair_offset[-1])

    def __eq__(self, other):
        return len(self) == len(other) and all(a == b for a, b in zip(self, other))

    __hash__ = None


class Engine:
    """One device context (stream + device buffers) of the engine."""

    def __init__(self, device: int = 0, mem_budget: int = 0):
        self.lib = library()
        h = C.c_void_p()
        rc = self.lib.dcns_ctx_create(device, mem_budget, C.byref(h))
        if rc != 0:
            raise DcnsError(rc, "could not create a context on cuda:%d (the engine needs an sm_103a GPU)" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.dcns_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def _check(self, rc):
        if rc != 0:
            raise DcnsError(rc, self.lib.dcns_last_error(self.h).decode(errors="replace"))

    @property
    def stream(self) -> int:
        return int(self.lib.dcns_ctx_stream(self.h) or 0)

    def set_lanes(self, lanes: int, bins: int):
        """Concurrent lanes and work bins for batches of at least 4096 pairs (results do not depend on them)."""
        self._check(self.lib.dcns_ctx_set_lanes(self.h, int(lanes), int(bins)))

    def autotune(self, batch, mode=MODE_ONE_GAP, **kw) -> dict:
        """Times the resident batch under candidate lane/bin shapes and keeps the fastest (results are unchanged)."""
        lanes, bins, ratio = C.c_int(), C.c_int(), C.c_double()
        self._check(self.lib.dcns_autotune(self.h, batch, C.byref(params(**kw)), mode, C.byref(lanes),
                                           C.byref(bins), C.byref(ratio)))
        return self.tuning()

    def tuning(self) -> dict:
        """The context's kernel shapes: pipeline shape, scan tiling, 2-piece warps and the per-bin x-drop forms."""
        t = Tuning()
        self._check(self.lib.dcns_get_tuning(self.h, C.byref(t)))
        return t.as_dict()

    def last_stats(self) -> dict:
        s = Stats()
        self._check(self.lib.dcns_last_stats(self.h, C.byref(s)))
        return s.as_dict()

    # -------------------------------------------------------------- whole path
    def align_pairs(self, pairs, mode=MODE_ONE_GAP, **kw):
        """Align many independent (seq1 codes, seq2 codes) pairs; returns one fragment list per pair."""
        arr, keep = _pairs(pairs)
        p = params(**kw)
        res = C.POINTER(Results)()
        self._check(self.lib.dcns_align_pairs(self.h, arr, len(keep), C.byref(p), mode, C.byref(res)))
        try:
            return _unpack(res)
        finally:
            self.lib.dcns_results_free(res)

    def prepare(self, pairs):
        """The dcns_pair table of a batch of host sequences (pointers to them, no copy), for align_prepared: the
        form a C or C++ caller already holds, so timing align_prepared times the C call itself."""
        return _pairs(pairs)

    def align_prepared(self, prepared, mode=MODE_ONE_GAP, **kw):
        """align_pairs on a prepare()d table: the sequences are read from host memory by dcns_align_pairs."""
        arr, keep = prepared
        p = params(**kw)
        res = C.POINTER(Results)()
        self._check(self.lib.dcns_align_pairs(self.h, arr, len(keep), C.byref(p), mode, C.byref(res)))
        try:
            return _unpack(res)
        finally:
            self.lib.dcns_results_free(res)

    def align_weighted(self, pairs, weights, cats, pieces=2, **kw):
        """weighted1Gap (pieces=1) / weighted2Gaps (pieces=2): weights[k] = category id per base of pair k's seq1,
        cats = [(match, mismatch, open1, ext1, open2, ext2, zdrop), ...]."""
        arr, keep = _pairs(pairs)
        wt = np.concatenate([np.asarray(w, np.int16).reshape(-1) for w in weights]) if weights else np.zeros(1, np.int16)
        if wt.size == 0:
            wt = np.zeros(1, np.int16)
        ct = np.ascontiguousarray(cats, np.int32).reshape(-1, 7)
        p = params(**kw)
        res = C.POINTER(Results)()
        self._check(self.lib.dcns_align_weighted(self.h, arr, len(keep), wt.ctypes.data_as(P16), ct.ctypes.data_as(_I32P),
                                                 len(ct), int(pieces), C.byref(p), C.byref(res)))
        try:
            return _unpack(res)
        finally:
            self.lib.dcns_results_free(res)

    def align_seeded(self, pairs, seeds, max_align_len=0, **kw):
        """cut2Gaps2's seeded 2-gap overload: seeds[k] = [(start1, end1, start2, end2), ...] 0-based, for pair k."""
        return self._seeded(self.lib.dcns_align_seeded, pairs, seeds, max_align_len=max_align_len, **kw)

    def align_xseeds(self, pairs, seeds, **kw):
        """The x-seed overload without maximumAlignLength (findSimilar...4.cpp:532): the 2-piece stage on the given
        x-seeds (seeds[k] = [(start1, end1, start2, end2), ...] 0-based, for pair k)."""
        return self._seeded(self.lib.dcns_align_xseeds, pairs, seeds, **kw)

    def _seeded(self, fn, pairs, seeds, **kw):
        arr, keep = _pairs(pairs)
        flat = np.zeros((max(1, sum(len(s) for s in seeds)), 4), np.int32)
        off = np.zeros(len(keep) + 1, np.int64)
        q = 0
        for k, sd in enumerate(seeds):
            for x in sd:
                flat[q] = x
                q += 1
            off[k + 1] = q
        p = params(**kw)
        res = C.POINTER(Results)()
        self._check(fn(self.h, arr, len(keep), flat.ctypes.data_as(_I32P), off.ctypes.data_as(_I64P), C.byref(p),
                       C.byref(res)))
        try:
            return _unpack(res)
        finally:
            self.lib.dcns_results_free(res)

    def align_one_to_many(self, ref, queries, mode=MODE_ONE_GAP, **kw):
        """One reference against many queries in one batched call, as the multi-species caller
        (getCnsForMultipleSpecies.cpp:126-135) runs pair by pair; the reference is staged and packed once."""
        ref = _codes(ref).reshape(-1)
        return self.align_pairs([(ref, q) for q in queries], mode, **kw)

    def upload(self, pairs):
        """Pack pairs into device memory once; returns a handle for align_resident."""
        arr, keep = _pairs(pairs)
        b = C.c_void_p()
        self._check(self.lib.dcns_batch_upload(self.h, arr, len(keep), C.byref(b)))
        return b

    def align_resident(self, batch, mode=MODE_ONE_GAP, **kw):
        """align_pairs on sequences already resident on the device (upload())."""
        p = params(**kw)
        res = C.POINTER(Results)()
        self._check(self.lib.dcns_align_batch(self.h, batch, C.byref(p), mode, C.byref(res)))
        try:
            return _unpack(res)
        finally:
            self.lib.dcns_results_free(res)

    def free_batch(self, batch):
        self.lib.dcns_batch_free(self.h, batch)

    def measure_scan_roofline(self) -> float:
        """GCUPS ceiling of the seed scan's instruction mix on this GPU, measured live."""
        g = C.c_double()
        self._check(self.lib.dcns_measure_scan_roofline(self.h, C.byref(g)))
        return float(g.value)

    def findSimilarFragmentsForPairedSequence(self, seq1, seq2, two_gap=False, **kw):
        """One pair, the reference's 1-gap (default) or 2-gap overload."""
        return self.align_pairs([(seq1, seq2)], MODE_TWO_GAP if two_gap else MODE_ONE_GAP, **kw)[0]

    # -------------------------------------------------------------- kernel-level
    def SmithWaterman(self, tasks, **kw):
        """SmithWaterman(ref, read, ...) per (ref, read) task -> int32 array [n, 3] (max, end1, end2)."""
        arr, keep = _pairs(tasks)
        out = np.zeros((max(1, len(keep)), 3), np.int32)
        self._check(self.lib.dcns_smith_waterman_batch(self.h, arr, len(keep), C.byref(params(**kw)),
                                                       out.ctypes.data_as(_I32P)))
        return out[:len(keep)]

    def _banded(self, fn, tasks, width, want_cigar, kw):
        arr, keep = _pairs(tasks)
        n = len(keep)
        out = np.zeros((max(1, n), width), np.int32)
        cap = (int(keep[1]["len1"].sum()) + int(keep[1]["len2"].sum()) + 4 * n + 4) if n else 4
        cig = np.zeros(cap, np.uint32)
        off = np.zeros(n + 1, np.int64)
        self._check(fn(self.h, arr, n, C.byref(params(**kw)), int(want_cigar), out.ctypes.data_as(_I32P),
                       cig.ctypes.data_as(_U32P), cap, off.ctypes.data_as(_I64P)))
        cigars = [[int(c) for c in cig[off[k]:off[k + 1]]] for k in range(n)]
        return out[:n], cigars

    def SemiGlobal_xextend(self, tasks, cigar=False, **kw):
        """x-drop extension per (seq1, seq2) task -> ([n, 6] = max, end1, end2, iii, jjj, ncigar; cigars)."""
        return self._banded(self.lib.dcns_xextend_batch, tasks, 6, cigar, kw)

    def SemiGlobal(self, tasks, cigar=False, **kw):
        """2-piece affine semi-global per task -> ([n, 4] = max, end1, end2, ncigar; cigars)."""
        return self._banded(self.lib.dcns_semiglobal_batch, tasks, 4, cigar, kw)

    def slidingWindowAlignment(self, seqs, **kw):
        """Per-window scores of seqs[0] against each other sequence: (score [n-1, n_windows], max [n-1, n_windows])."""
        keep = [_codes(s) for s in seqs]
        ptrs = (_I8P * len(keep))(*[s.ctypes.data_as(_I8P) for s in keep])
        lens = np.array([len(s) for s in keep], np.int32)
        p = params(**kw)
        nw = (len(keep[0]) + p.step - 1) // p.step
        sc = np.zeros((max(1, len(keep) - 1), max(nw, 1)), np.float64)
        mx = np.zeros_like(sc, dtype=np.int32)
        self._check(self.lib.dcns_sliding_window(self.h, ptrs, lens.ctypes.data_as(_I32P), len(keep), C.byref(p),
                                                 sc.ctypes.data_as(_F64P), mx.ctypes.data_as(_I32P)))
        return sc[:len(keep) - 1, :nw], mx[:len(keep) - 1, :nw]

    # -------------------------------------------------------------- serving loop
    def serve_start(self, mode=MODE_ONE_GAP, max_inflight=256, workers=3, batch_cells=0, admit_bytes=0, **kw):
        """Starts the continuous-batching loop (workers: 1..8; batch_cells / admit_bytes: the batch caps in predicted
        level-0 scan cells and device bytes, 0 = defaults)."""
        self._check(self.lib.dcns_serve_set_shape(self.h, int(workers), int(batch_cells), int(admit_bytes)))
        self._serve_params = params(**kw)
        self._check(self.lib.dcns_serve_start(self.h, C.byref(self._serve_params), mode, max_inflight))

    def cancel(self, ticket: int):
        self._check(self.lib.dcns_cancel(self.h, ticket))

    def poll(self, ticket: int):
        """The result if done, None while pending (raises on a failed or unknown ticket)."""
        res = C.POINTER(Results)()
        rc = self.lib.dcns_poll(self.h, ticket, C.byref(res))
        if rc == -6:
            return None
        self._check(rc)
        try:
            return _unpack(res)[0]
        finally:
            self.lib.dcns_results_free(res)

    def serve_stats(self) -> dict:
        s = ServingStats()
        self._check(self.lib.dcns_serve_stats(self.h, C.byref(s)))
        return s.as_dict()

    def submit(self, seq1, seq2) -> int:
        arr, keep = _pairs([(seq1, seq2)])
        t = C.c_uint64()
        self._check(self.lib.dcns_submit(self.h, arr, C.byref(t)))
        return int(t.value)

    def wait(self, ticket: int, timeout_ms: int = 600000):
        res = C.POINTER(Results)()
        self._check(self.lib.dcns_serve_wait(self.h, ticket, timeout_ms, C.byref(res)))
        try:
            return _unpack(res)[0]
        finally:
            self.lib.dcns_results_free(res)

    def serve_stop(self):
        self._check(self.lib.dcns_serve_stop(self.h))


def load(device: int = 0, mem_budget: int = 0) -> Engine:
    """Build (if needed) and open an engine on cuda:<device>."""
    build()
    return Engine(device, mem_budget)
