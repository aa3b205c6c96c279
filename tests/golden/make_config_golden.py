"""Generates tests/golden/configs.npz: what the UNMODIFIED dCNS reference (oracle/_ref/libdcns_ref.so, built from the
reference checkout by oracle/build_ref.sh) computes on the benchmark workloads themselves, as compact digests
(config_digest.py).  Run here, where the reference exists (about 40 CPU-minutes, spread over the host cores):

    python tests/golden/make_config_golden.py [processes]

Sections (inputs regenerated from dcns_gb300.workloads with their default seeds):
  c2p1  the 10,000-pair batched workload, cut1Gap (1-gap) path, every pair
  c2p2  its first 500 pairs, cut2Gaps (2-piece) path
  c4    the first 10,000 seeds of the extension-stress workload: the forward pass (no CIGAR) and the CIGAR pass
  c5p1  serving requests: the first 200 of the 2,000-request workload whose sequences are both at most 20 kb, 1-gap
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

N_C2, N_C2P2, N_C4, N_C5, N_C5_SEL, C5_MAX = 10000, 500, 10000, 2000, 200, 20000
_cache = {}


def workload(name):
    from dcns_gb300 import workloads as W
    if name not in _cache:
        if name == "c2":
            _cache[name] = W.config2(n_pairs=N_C2)
        elif name == "c4":
            _cache[name] = W.config4(n_seeds=N_C4)
        elif name == "c5":
            reqs = W.config5(n_requests=N_C5)
            idx = [i for i, (a, b) in enumerate(reqs) if max(len(a), len(b)) <= C5_MAX][:N_C5_SEL]
            _cache[name] = (np.array(idx, np.int32), [reqs[i] for i in idx])
    return _cache[name]


def job(args):
    section, lo, hi = args
    from oracle import oracle as O
    import config_digest as D
    ref = _cache.setdefault("ref", None) or O.Reference()
    _cache["ref"] = ref
    if section in ("c2p1", "c2p2"):
        pairs = workload("c2")[lo:hi]
        return section, lo, D.pair_digests([ref.find(a, b, two_gap=section == "c2p2") for a, b in pairs])
    if section == "c5p1":
        pairs = workload("c5")[1][lo:hi]
        return section, lo, D.pair_digests([ref.find(a, b) for a, b in pairs])
    tasks = workload("c4")[lo:hi]
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
    import config_digest as D
    jobs = [("c2p1", lo, min(lo + 50, N_C2)) for lo in range(0, N_C2, 50)]
    jobs += [("c2p2", lo, min(lo + 25, N_C2P2)) for lo in range(0, N_C2P2, 25)]
    jobs += [("c4", lo, min(lo + 1000, N_C4)) for lo in range(0, N_C4, 1000)]
    jobs += [("c5p1", lo, min(lo + 10, N_C5_SEL)) for lo in range(0, N_C5_SEL, 10)]
    t0 = time.time()
    parts = {}
    with mp.get_context("spawn").Pool(procs) as pool:
        for k, (sec, lo, res) in enumerate(pool.imap_unordered(job, jobs)):
            parts.setdefault(sec, []).append((lo, res))
            if k % 25 == 0:
                print(f"{k + 1}/{len(jobs)} jobs, {time.time() - t0:.0f} s", flush=True)
    out = {}
    for sec in ("c2p1", "c2p2", "c5p1"):
        chunks = [r for _, r in sorted(parts[sec], key=lambda x: x[0])]
        out[sec + "_nfrag"] = np.concatenate([c[0] for c in chunks])
        out[sec + "_hash"] = np.concatenate([c[1] for c in chunks])
        out[sec + "_pe"] = np.concatenate([c[2] for c in chunks])
    chunks = [r for _, r in sorted(parts["c4"], key=lambda x: x[0])]
    out["c4_nocigar"] = np.concatenate([c[0] for c in chunks])
    out["c4_cigar"] = np.concatenate([c[1] for c in chunks])
    out["c4_cigar_hash"] = np.concatenate([c[2] for c in chunks])
    out["c2_inputs"] = np.array(D.inputs_hash(workload("c2")))
    out["c4_inputs"] = np.array(D.inputs_hash(workload("c4")))
    idx, sel = workload("c5")
    out["c5_index"] = idx
    out["c5_inputs"] = np.array(D.inputs_hash(sel))
    dst = os.path.join(HERE, "configs.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes;", int(out["c2p1_nfrag"].sum()), "1-gap fragments (10,000 pairs),",
          int(out["c2p2_nfrag"].sum()), "2-gap,", int(out["c5p1_nfrag"].sum()), "serving;", f"{time.time() - t0:.0f} s")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count() or 1)
