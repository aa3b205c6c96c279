"""Generates tests/golden/long_digests.npz: digests (digest.py) of what the reference computes on the two long-pair
shapes, where its dense traceback matrix of (L1+1)(L2+1) bytes per alignment does not fit in memory.  The
reference runs unmodified except for that matrix: oracle/_ref/libdcns_ref_lazy.so links oracle/lazy_matrix.cpp,
which stores only the cells an alignment touches and keeps the matrix's get/set/reset semantics.  Run here, where the
reference exists (about 25 minutes on 8 cores):

    python tests/golden/make_long_digests.py [processes]

Sections (inputs regenerated from dcns_gb300.workloads with their default seeds):
  long_1gap           the first 4 pairs of the 200 kb long-pair workload, whole (200 kb x ~234 kb), cut1Gap path;
                      computed by the reference and by the oracle restatement, which must agree
  serving_long_1gap   the first 20 requests of the 2,000-request serving workload whose sequences are both longer
                      than 42.5 kb after masking (its 50-100 kb class), cut1Gap path, by the reference
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

N_LONG, N_SERVING, N_SERVING_LONG, LONG_MIN = 4, 2000, 20, 42500
_cache = {}


def long_pairs():
    from dcns_gb300 import workloads as W
    if "long" not in _cache:
        _cache["long"] = W.long_pairs_200kb(n_pairs=N_LONG)
    return _cache["long"]


def serving_long():
    """(indices into the serving workload, requests) of its first N_SERVING_LONG long requests."""
    from dcns_gb300 import workloads as W
    if "serving" not in _cache:
        reqs = W.serving_requests(n_requests=N_SERVING)
        idx = [i for i, (a, b) in enumerate(reqs) if min(len(a), len(b)) > LONG_MIN][:N_SERVING_LONG]
        _cache["serving"] = (np.array(idx, np.int32), [reqs[i] for i in idx])
    return _cache["serving"]


def job(args):
    section, who, k = args
    from oracle import oracle as O
    import digest as D
    if section == "long_1gap":
        a, b = long_pairs()[k]
    else:
        a, b = serving_long()[1][k]
    t = time.time()
    frs = O.Reference(lazy=True).find(a, b) if who == "reference" else O.Oracle().find(a, b)[0]
    return section, who, k, D.pair_digests([frs]), time.time() - t


def main(procs):
    from oracle import oracle as O
    import digest as D
    O.build()
    jobs = [("long_1gap", who, k) for k in range(N_LONG) for who in ("reference", "oracle")]
    jobs += [("serving_long_1gap", "reference", k) for k in range(N_SERVING_LONG)]
    t0 = time.time()
    res = {}
    with mp.get_context("spawn").Pool(procs) as pool:
        for sec, who, k, dg, dt in pool.imap_unordered(job, jobs):
            res[(sec, who, k)] = dg
            print(f"{sec} {who} #{k}: {int(dg[0][0])} fragments, {dt:.0f} s (total {time.time() - t0:.0f} s)",
                  flush=True)
    out = {}
    for sec, n in (("long_1gap", N_LONG), ("serving_long_1gap", N_SERVING_LONG)):
        parts = [res[(sec, "reference", k)] for k in range(n)]
        out[sec + "_nfrag"] = np.concatenate([p[0] for p in parts])
        out[sec + "_hash"] = np.concatenate([p[1] for p in parts])
        out[sec + "_pe"] = np.concatenate([p[2] for p in parts])
    for k in range(N_LONG):
        r, o = res[("long_1gap", "reference", k)], res[("long_1gap", "oracle", k)]
        assert r[0][0] == o[0][0] and r[1][0] == o[1][0], f"oracle and reference differ on long pair {k}"
        assert abs(r[2][0] - o[2][0]).max() <= 1e-12 * max(abs(r[2][0]).max(), 1e-300), k
    out["long_inputs"] = np.array(D.inputs_hash(long_pairs()))
    idx, sel = serving_long()
    out["serving_long_index"] = idx
    out["serving_long_inputs"] = np.array(D.inputs_hash(sel))
    dst = os.path.join(HERE, "long_digests.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes;", int(out["long_1gap_nfrag"].sum()), "long-pair fragments,",
          int(out["serving_long_1gap_nfrag"].sum()), "long serving fragments;", f"{time.time() - t0:.0f} s")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count() or 1)
