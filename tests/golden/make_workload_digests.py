"""Generates tests/golden/workload_digests.npz: what the UNMODIFIED dCNS reference (oracle/_ref/libdcns_ref.so, built
from the reference checkout by oracle/build_ref.sh) computes on the benchmark workloads themselves, as compact
digests (digest.py).  Run here, where the reference exists (about 40 CPU-minutes, spread over the host cores):

    python tests/golden/make_workload_digests.py [processes]

Sections (inputs regenerated from dcns_gb300.workloads with their default seeds):
  batch_1gap    the 10,000-pair batched workload, cut1Gap (1-gap) path, every pair
  batch_2gap    its first 500 pairs, cut2Gaps (2-piece) path
  seeds         the first 10,000 seeds of the extension-stress workload: the forward pass (no CIGAR) and the CIGAR pass
  serving_1gap  serving requests: the first 200 of the 2,000-request workload whose sequences are both at most
                20 kb, 1-gap
                (the longer requests need the reference's dense traceback matrix of (L1+1)(L2+1) bytes per extension)
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

N_BATCH, N_BATCH_2GAP, N_SEEDS, N_SERVING, N_SERVING_SEL, SERVING_MAX = 10000, 500, 10000, 2000, 200, 20000
_cache = {}


def workload(name):
    from dcns_gb300 import workloads as W
    if name not in _cache:
        if name == "batch":
            _cache[name] = W.batched_pairs(n_pairs=N_BATCH)
        elif name == "seeds":
            _cache[name] = W.extension_seeds(n_seeds=N_SEEDS)
        elif name == "serving":
            reqs = W.serving_requests(n_requests=N_SERVING)
            idx = [i for i, (a, b) in enumerate(reqs) if max(len(a), len(b)) <= SERVING_MAX][:N_SERVING_SEL]
            _cache[name] = (np.array(idx, np.int32), [reqs[i] for i in idx])
    return _cache[name]


def job(args):
    section, lo, hi = args
    from oracle import oracle as O
    import digest as D
    ref = _cache.setdefault("ref", None) or O.Reference()
    _cache["ref"] = ref
    if section in ("batch_1gap", "batch_2gap"):
        pairs = workload("batch")[lo:hi]
        return section, lo, D.pair_digests([ref.find(a, b, two_gap=section == "batch_2gap") for a, b in pairs])
    if section == "serving_1gap":
        pairs = workload("serving")[1][lo:hi]
        return section, lo, D.pair_digests([ref.find(a, b) for a, b in pairs])
    tasks = workload("seeds")[lo:hi]
    nc = np.zeros((len(tasks), 3), np.int32)
    cg = np.zeros((len(tasks), 5), np.int32)
    ch = np.zeros(len(tasks), np.uint64)
    for k, (a, b) in enumerate(tasks):
        e = ref.xextend(a, b)
        nc[k] = (e["score"], e["end1"], e["end2"])
        e = ref.xextend(a, b, cigar=True)
        cg[k] = (e["score"], e["end1"], e["end2"], e["iii"], e["jjj"])
        ch[k] = D.cigar_hash(e["cigar"])
    return section, lo, (nc, cg, ch)


def main(procs):
    import digest as D
    jobs = [("batch_1gap", lo, min(lo + 50, N_BATCH)) for lo in range(0, N_BATCH, 50)]
    jobs += [("batch_2gap", lo, min(lo + 25, N_BATCH_2GAP)) for lo in range(0, N_BATCH_2GAP, 25)]
    jobs += [("seeds", lo, min(lo + 1000, N_SEEDS)) for lo in range(0, N_SEEDS, 1000)]
    jobs += [("serving_1gap", lo, min(lo + 10, N_SERVING_SEL)) for lo in range(0, N_SERVING_SEL, 10)]
    t0 = time.time()
    parts = {}
    with mp.get_context("spawn").Pool(procs) as pool:
        for k, (sec, lo, res) in enumerate(pool.imap_unordered(job, jobs)):
            parts.setdefault(sec, []).append((lo, res))
            if k % 25 == 0:
                print(f"{k + 1}/{len(jobs)} jobs, {time.time() - t0:.0f} s", flush=True)
    out = {}
    for sec in ("batch_1gap", "batch_2gap", "serving_1gap"):
        chunks = [r for _, r in sorted(parts[sec], key=lambda x: x[0])]
        out[sec + "_nfrag"] = np.concatenate([c[0] for c in chunks])
        out[sec + "_hash"] = np.concatenate([c[1] for c in chunks])
        out[sec + "_pe"] = np.concatenate([c[2] for c in chunks])
    chunks = [r for _, r in sorted(parts["seeds"], key=lambda x: x[0])]
    out["seeds_nocigar"] = np.concatenate([c[0] for c in chunks])
    out["seeds_cigar"] = np.concatenate([c[1] for c in chunks])
    out["seeds_cigar_hash"] = np.concatenate([c[2] for c in chunks])
    out["batch_inputs"] = np.array(D.inputs_hash(workload("batch")))
    out["seeds_inputs"] = np.array(D.inputs_hash(workload("seeds")))
    idx, sel = workload("serving")
    out["serving_index"] = idx
    out["serving_inputs"] = np.array(D.inputs_hash(sel))
    dst = os.path.join(HERE, "workload_digests.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes;", int(out["batch_1gap_nfrag"].sum()),
          "1-gap fragments (10,000 pairs),", int(out["batch_2gap_nfrag"].sum()), "2-gap,",
          int(out["serving_1gap_nfrag"].sum()), "serving;", f"{time.time() - t0:.0f} s")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count() or 1)
