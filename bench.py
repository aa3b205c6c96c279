#!/usr/bin/env python
"""Benchmark of the batched CNS pair-alignment hot path (cut1Gap: seed scan + recursion + x-drop extension).

Workload: 10,000 independent pairs with log-normal lengths (median 3 kb, sigma 0.8, clipped to 0.5-20 kb) and
Poisson(8) planted 30-300 bp conserved segments at 70-95 % identity, 1 % indels, 15 % masked runs (seeded synthetic
data with the batched configuration's shapes).  One step = one pass of the pipeline over the whole batch.

Reported (one JSON line, rank 0):
  value   algorithmic GCUPS of the whole pipeline with the sequences resident in HBM (dcns_align_batch)
  e2e     the same through the public call with host buffers (dcns_align_pairs): H2D of the codes, the pipeline,
          and the D2H of the fragments inside the timed region
  roofline  the seed-scan kernel (dominant) against the live-measured integer-issue ceiling of its instruction mix
  cpu_baseline  the oracle restatement of the reference over all host cores on a fixed sample of the workload (every
          k-th pair, 64 per thread)
  per_pair_launch, serving  the one-pair-per-call form and the continuous-batching loop (p50/p99) for comparison
  two_gap, long_pairs, seeded_chromosome, extension_seeds  the other benchmark configurations (the cut2Gaps path,
          whole 200 kb pairs, cut2Gaps2's seeded overload on a whole 200 kb pair with no length cap, 1,000,000
          extension seeds), each with its kernel figures, its own CPU baseline and clock record

`--impl reference` times the reference's CPU implementation of the path instead (the oracle restatement, since the
reference sources are not present on the GPU host), with every host core, each step one pass over the same fixed
sample the cpu_baseline above times.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GCUPS & pairs/s, batched vs per-pair launch on 1 GB300, bit-exact; p99 latency"


def workload_name(n, mode):
    path = "cut1Gap" if mode == 1 else "cut2Gaps"
    return f"batched seed scan + extension: {n:,} pairs, log-normal 0.5-20 kb ({path} path)"


L2_NOTE = ("GPU steps: L2 (129 MB) flushed by a 256 MB device write before every timed step; CPU steps: host caches "
           "not flushed")


def bench_config(n, mode, world):
    """The workload keys shared by both arms' JSON lines (same dict, so the two arms name the same configuration)."""
    return {"workload": workload_name(n, mode), "pairs": n, "mode": mode, "parallelism": f"replicas x{world}",
            "l2": L2_NOTE}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=10000)
    ap.add_argument("--mode", type=int, default=1, help="1 = cut1Gap (1-gap), 2 = cut2Gaps (2-piece)")
    ap.add_argument("--ext-seeds", type=int, default=1000000, help="seeds of the extension-stress line")
    ap.add_argument("--no-extras", action="store_true", help="skip the per-pair and serving comparisons")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default pipeline shape (4 lanes, 4 bins, ratio 0.6) instead of timing "
                         "candidate shapes first (profiling runs: no trial calls before the warm-up)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def workload(n_pairs, rank=0):
    from dcns_gb300 import workloads as W
    from dcns_gb300.ranks import shard_seed
    return W.batched_pairs(n_pairs=n_pairs, seed=shard_seed(rank))


# DRAM bytes per algorithmic cell of the level-0 scan launch: ncu, 3,000 pairs of this workload, 18.51 MB read and 0
# written for 161.25 G cells (profiles/scan_kernel_batched_3000pairs.md); traffic grows with the cells.
SCAN_DRAM_BYTES_PER_CELL = 18.51392e6 / 161254407231


def level0_cells(pairs, window=38, step=8):
    """Algorithmic cells of the level-0 scan (every window of every pair against its whole reference)."""
    tot = 0
    for a, b in pairs:
        n1, n2 = len(a), len(b)
        istar = 1 if n2 - window < 0 else (n2 - window) // step + 1
        nwin = istar + (0 if istar * step > n2 else 1)
        nfast = min(nwin, (n2 + step - 1) // step) if n1 > 0 else 0
        tot += n1 * sum(max(0, min(window, n2 - w * step)) for w in range(nfast))
    return tot


def cells_of(st):
    return st["cells_scan"] + st["cells_scan_reverse"] + st["cells_xdrop"] + st["cells_semiglobal"]


def cpu_sample(pairs, threads, per_thread=64):
    """A fixed sample of the workload for the CPU timings: every k-th pair (so its length mix is the workload's),
    per_thread pairs per host thread, handed out longest first so that the shared work counter does not end on a long
    pair.  The same sample every step and in both arms."""
    n = max(1, min(len(pairs), per_thread * threads))
    stride = len(pairs) / n
    idx = sorted({int(i * stride) for i in range(n)}, key=lambda i: (-len(pairs[i][0]) * len(pairs[i][1]), i))
    desc = (f"every {stride:.2f}th pair of the {len(pairs):,}-pair workload ({len(idx)} pairs, longest first), "
            f"{threads} threads")
    return [pairs[i] for i in idx], desc


def cpu_baseline(sample, desc, mode, threads):
    """One pass of the oracle restatement of the reference over the sample, on `threads` host threads."""
    from oracle import oracle as O
    O.build()
    orc = O.Oracle()
    t = time.perf_counter()
    _, _, cells = orc.find_batch(sample, two_gap=(mode == 2), threads=threads)
    dt = max(time.perf_counter() - t, 1e-6)
    tot = cells["scan"] + cells["scan_rev"] + cells["xdrop"] + cells["semiglobal"]
    return {"value": tot / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port", "pairs_per_s": len(sample) / dt,
            "seconds": dt, "sample": desc}


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path (the oracle restatement: the reference sources do not travel
    to the GPU host) on every host thread, each step one pass over the fixed sample that the GPU arm's cpu_baseline
    also times; warm-up steps pass over its first eighth."""
    if rank != 0:
        return
    pairs = workload(args.pairs)
    threads = host_threads()
    sample, desc = cpu_sample(pairs, threads)
    for _ in range(args.warmup):
        cpu_baseline(sample[:max(1, len(sample) // 8)], desc, args.mode, threads)
    steps = [cpu_baseline(sample, desc, args.mode, threads) for _ in range(args.steps)]
    val = statistics.median(s["value"] for s in steps)
    cb = dict(steps[-1], value=val, seconds=statistics.median(s["seconds"] for s in steps))
    line = {"impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "GCUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * statistics.median(s["seconds"] for s in steps), 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded)", "config": bench_config(args.pairs, args.mode, world),
            "pairs_per_s": round(statistics.median(s["pairs_per_s"] for s in steps), 2),
            "cpu_baseline": cb, "e2e": {"value": round(val, 4), "unit": "GCUPS", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def hbm_peak():
    """The measured copy bandwidth of the GB300s (MEASURED_PEAKS.json), else the stated fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def line_two_gap(eng, timed, pairs, threads, gpu, n=2000, steps=3):
    """cut2Gaps (2-piece) path over the first n pairs of the batched workload, resident on the device: GCUPS of the
    whole path, and the semi-global DP kernel (sg_kernel) and its traceback alone (CUDA events)."""
    sub = pairs[:n]
    b = eng.upload(sub)
    eng.align_resident(b, 2)
    tot_ms, cells, sg_ms, sgtb_ms, sg_cells, sg_bytes = 0.0, 0, 0.0, 0.0, 0, 0
    with ClockSampler(gpu) as clk:
        for _ in range(steps):
            _, t = timed(lambda: eng.align_resident(b, 2))
            st = eng.last_stats()
            tot_ms += t
            cells += cells_of(st)
            sg_ms += st["ms_sg_kernel"]
            sgtb_ms += st["ms_sg_tb_kernel"]
            sg_cells += st["cells_semiglobal"]
            sg_bytes += st["bytes_codes_sg"]
    eng.free_batch(b)
    sample, desc = cpu_sample(sub, threads, per_thread=32)
    return {"workload": f"batched pairs, first {n:,}, cut2Gaps path (2-piece semi-global after the 1-gap seeds)",
            "value": round(cells / (tot_ms * 1e-3) / 1e9, 3), "unit": "GCUPS", "steps": steps,
            "ms_per_step": round(tot_ms / steps, 2), "pairs_per_s": round(n * steps / (tot_ms * 1e-3), 1),
            "sg_kernel": {"ms_per_step": round(sg_ms / steps, 2), "gcups": round(sg_cells / (sg_ms * 1e-3) / 1e9, 2),
                          "traceback_ms_per_step": round(sgtb_ms / steps, 2),
                          "codes_gb_per_s": round(sg_bytes / (sg_ms * 1e-3) / 1e9, 2),
                          "timing": "CUDA events around each semi-global DP and traceback launch"},
            "cpu_baseline": cpu_baseline(sample, desc, 2, threads), "clocks": clk.summary()}


def line_long_pairs(eng, timed, threads, gpu, scan_peak, n=8, steps=2, cpu_query=2000):
    """Long pairs: n whole 200 kb x ~234 kb pairs (the long-pair workload's first n), cut1Gap path, resident; the
    seed-scan kernel's GCUPS against the live integer-issue ceiling.  The CPU baseline aligns the first cpu_query bases
    of each query of the first `threads` pairs against their whole references (one slice per thread)."""
    from dcns_gb300 import workloads as W
    pairs = W.long_pairs_200kb(n_pairs=max(n, threads))
    b = eng.upload(pairs[:n])
    eng.align_resident(b, 1)
    tot_ms, cells, scan_ms, scan_cells, nfrag = 0.0, 0, 0.0, 0, 0
    with ClockSampler(gpu) as clk:
        for _ in range(steps):
            res, t = timed(lambda: eng.align_resident(b, 1))
            st = eng.last_stats()
            tot_ms += t
            cells += cells_of(st)
            scan_ms += st["ms_scan_kernel"]
            scan_cells += st["cells_scan"]
            nfrag = sum(len(f) for f in res)
    eng.free_batch(b)
    from oracle import oracle as O
    O.build()
    slices = [(a, q[:cpu_query]) for a, q in pairs[:threads]]
    t0 = time.perf_counter()
    _, _, cc = O.Oracle().find_batch(slices, threads=threads)
    dt = time.perf_counter() - t0
    cpu_cells = cc["scan"] + cc["scan_rev"] + cc["xdrop"] + cc["semiglobal"]
    achieved = scan_cells / (scan_ms * 1e-3) / 1e9
    return {"workload": f"long pairs: {n} whole pairs of 200 kb x ~234 kb (GC 45 %, 500 planted segments, 5 "
                        f"duplicated 2-10 kb blocks), cut1Gap path",
            "value": round(cells / (tot_ms * 1e-3) / 1e9, 3), "unit": "GCUPS", "steps": steps,
            "ms_per_step": round(tot_ms / steps, 2), "pairs_per_s": round(n * steps / (tot_ms * 1e-3), 2),
            "fragments": nfrag,
            "scan_roofline": {"kernel": "scan_kernel<38> (row-chunked)", "achieved": round(achieved, 1),
                              "peak": round(scan_peak, 1), "unit": "GCUPS", "frac": round(achieved / scan_peak, 4),
                              "share_of_step": round(scan_ms / tot_ms, 4)},
            "cpu_baseline": {"value": cpu_cells / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "seconds": dt, "sample": f"the first {cpu_query} bases of the query of each of the first "
                                                      f"{len(slices)} pairs against its whole 200 kb reference, one "
                                                      f"slice per thread"},
            "clocks": clk.summary()}


def line_seeded_chromosome(eng, timed, threads, gpu, steps=3, n_seeds=16, cpu_seeds=None, cpu_len=20000):
    """cut2Gaps2's seeded 2-gap overload at chromosome scale: one whole 200 kb x ~234 kb pair of the long-pair workload
    with maximumAlignLength unlimited (the reference's driver caps it at 140 kb for its dense traceback matrix).  The
    x-seeds are the pair's first n_seeds cut1Gap fragments (as cut2Gaps2 reads them from a SAM file of earlier
    alignments).  C ABI call on host buffers (upload and result download in every step); the 2-piece kernels'
    GCUPS, and the device memory the call's buffers hold.  The CPU baseline runs the oracle port on a sample of the
    pair's leading part (a whole-pair seed takes minutes on one core), one seed per thread."""
    from concurrent.futures import ThreadPoolExecutor
    from dcns_gb300 import workloads as W
    import dcns_gb300 as D
    a, b = W.long_pairs_200kb(n_pairs=1)[0]
    frs = eng.align_pairs([(a, b)], 1)[0][:n_seeds]
    seeds = [(f.start1 - 1, f.end1 - 1, f.start2 - 1, f.end2 - 1) for f in frs]
    # a context of its own, so that its buffers are this call's alone (device_bytes)
    own = D.Engine(gpu)
    own.align_seeded([(a, b)], [seeds], max_align_len=0)
    tot_ms, cells, sg_ms, tb_ms, nfrag, dev = 0.0, 0, 0.0, 0.0, 0, 0
    with ClockSampler(gpu) as clk:
        for _ in range(steps):
            res, t = timed(lambda: own.align_seeded([(a, b)], [seeds], max_align_len=0))
            st = own.last_stats()
            tot_ms += t
            cells += st["cells_semiglobal"]
            sg_ms += st["ms_sg_kernel"]
            tb_ms += st["ms_sg_tb_kernel"]
            nfrag = len(res[0])
            dev = max(dev, st["bytes_device"])
    own.close()
    # CPU: the same kind of call on the pair's first cpu_len bases of each sequence (a whole-pair seed takes about two
    # minutes of one core), one x-seed per thread, cells counted by the oracle
    from oracle import oracle as O
    O.build()
    ca, cb = a[:cpu_len], b[:int(cpu_len * len(b) / len(a))]
    sample = [s for s in seeds if s[1] < len(ca) - 1 and s[3] < len(cb) - 1][:cpu_seeds or threads]
    orc = O.Oracle()

    def one(sd):
        return orc.find_seeded(ca, cb, [sd], 1 << 30, with_cells=True)[1]["semiglobal"]

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max(1, len(sample))) as ex:
        cpu_cells = sum(ex.map(one, sample))
    dt = time.perf_counter() - t0
    return {"workload": f"cut2Gaps2 seeded overload: one whole 200 kb x {len(b) // 1000} kb pair, {len(seeds)} x-seeds "
                        f"(its first cut1Gap fragments), maximumAlignLength unlimited",
            "value": round(cells / (tot_ms * 1e-3) / 1e9, 3), "unit": "GCUPS", "steps": steps,
            "ms_per_step": round(tot_ms / steps, 2), "fragments": nfrag,
            "sg_kernel": {"ms_per_step": round(sg_ms / steps, 2), "gcups": round(cells / (sg_ms * 1e-3) / 1e9, 2),
                          "traceback_ms_per_step": round(tb_ms / steps, 2)},
            "device_bytes": int(dev),
            "device_memory_note": "device buffers the call holds (sequences, DP codes of one DP per seed at 1 byte "
                                  "per band cell, boundary rows); the reference's dense traceback matrix for this "
                                  f"pair would be {(len(a) + 1) * (len(b) + 1) / 1e9:.0f} GB",
            "cpu_baseline": {"value": cpu_cells / dt / 1e9, "unit": "GCUPS", "cores": len(sample), "kind": "port",
                             "seconds": dt,
                             "sample": f"the same call on the pair's first {len(ca):,} x {len(cb):,} bases, its first "
                                       f"{len(sample)} x-seeds there, one per thread"},
            "clocks": clk.summary()}


def _seed_chunk(c):
    from dcns_gb300 import workloads as W
    return W.extension_seeds(n_seeds=10000, seed=20261207 + c)


def extension_workload(n):
    """n extension-stress seeds: chunks of 10,000 drawn by the workload's generator with seeds 20261207 + c (chunk 0
    is the reference-digested set), generated in a process pool."""
    import multiprocessing as mp
    chunks = (n + 9999) // 10000
    with mp.get_context("spawn").Pool(max(1, min(host_threads(), chunks))) as pool:
        parts = pool.map(_seed_chunk, range(chunks))
    return [t for p in parts for t in p][:n]


def line_extension_seeds(eng, n, threads, gpu, steps=3):
    """Extension stress: n seeds through x_extend_seed's two SemiGlobal_xextend passes (forward, then with the
    traceback: 4-bit direction codes written, the traceback walk, CIGARs packed on the device) by the C ABI call on
    host buffers, so each step includes the upload of the codes and the download of the results."""
    import ctypes as C
    import dcns_gb300 as D
    t0 = time.perf_counter()
    tasks = extension_workload(n)
    gen_s = time.perf_counter() - t0
    arr, keep = eng.prepare(tasks)
    out = np.zeros((n, 6), np.int32)
    cap = int(keep[1]["len1"].sum()) + int(keep[1]["len2"].sum()) + 4 * n + 4
    cig = np.zeros(cap, np.uint32)
    off = np.zeros(n + 1, np.int64)
    p = D.params()
    lib = eng.lib

    def call(want):
        rc = lib.dcns_xextend_batch(eng.h, arr, n, C.byref(p), want, out.ctypes.data_as(D._I32P),
                                    cig.ctypes.data_as(D._U32P), cap, off.ctypes.data_as(D._I64P))
        if rc != 0:
            raise D.DcnsError(rc, lib.dcns_last_error(eng.h).decode())
        return eng.last_stats()

    call(0), call(1)
    wall, cells, k_ms, tb_ms, code_bytes, path_cells = 0.0, 0, 0.0, 0.0, 0, 0
    with ClockSampler(gpu) as clk:
        for _ in range(steps):
            t = time.perf_counter()
            s0 = call(0)
            s1 = call(1)
            wall += time.perf_counter() - t
            cells += s0["cells_xdrop"] + s1["cells_xdrop"]
            k_ms += s1["ms_xdrop_kernel"]
            tb_ms += s1["ms_xdrop_tb_kernel"]
            code_bytes += s1["bytes_codes_xdrop"]
            path_cells += int((cig[:off[-1]] >> 4).sum())
    peak, kind = hbm_peak()
    codes_gbs = code_bytes / (k_ms * 1e-3) / 1e9
    tb_gbs = path_cells * 0.5 / (tb_ms * 1e-3) / 1e9
    per_thread = 5000  # about 10 s of both passes on a Grace core
    sample = tasks[::max(1, n // (per_thread * threads))][:per_thread * threads]
    from oracle import oracle as O
    O.build()
    t = time.perf_counter()
    _, _, cpu_cells = O.Oracle().xextend_batch(sample, threads=threads)
    dt = time.perf_counter() - t
    return {"workload": f"extension stress: {n:,} seeds (38 bp core, 50-2000 bp flanks at 50-98 % identity), both "
                        f"x_extend_seed passes per seed",
            "value": round(cells / wall / 1e9, 3), "unit": "GCUPS", "steps": steps,
            "ms_per_step": round(wall / steps * 1e3, 2), "seeds_per_s": round(n * steps / wall, 1),
            "e2e": "C ABI call on host buffers: upload of the codes and download of the results in every step",
            "xdrop_kernels": {"traceback_pass_level_kernels_ms": round(k_ms / steps, 2),
                              "traceback_kernels_ms": round(tb_ms / steps, 2),
                              "codes_written_gb_per_s": round(codes_gbs, 2),
                              "traceback_read_gb_per_s": round(tb_gbs, 2),
                              "hbm_peak_gb_per_s": peak, "peak_kind": kind,
                              "codes_frac_of_peak": round(codes_gbs / peak, 5),
                              "bytes": "codes: 4 bits per final-width band cell of the traceback pass; traceback: "
                                       "4 bits per path cell"},
            "generation_s": round(gen_s, 1),
            "cpu_baseline": {"value": cpu_cells / dt / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "seconds": dt, "sample": f"every {max(1, n // (per_thread * threads))}th seed "
                                                      f"({len(sample)} seeds), both passes, {threads} threads"},
            "clocks": clk.summary()}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import dcns_gb300
    from dcns_gb300 import ranks as R

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dcns_gb300.build()
    eng = dcns_gb300.Engine(local)
    stream = torch.cuda.ExternalStream(eng.stream)
    # each rank aligns its own shard of pairs (weak scaling: no data-path collective)
    pairs = workload(args.pairs, rank)
    n = len(pairs)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn):
        flush.fill_(1)  # L2 (129 MB) flushed between timed iterations
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1)

    # ---- value: resident sequences (pipeline shape chosen by the library's autotuner on this batch first)
    batch = eng.upload(pairs)
    tuned = dict(eng.tuning(), autotuned=False) if args.no_autotune else dict(eng.autotune(batch, args.mode),
                                                                               autotuned=True)
    for _ in range(max(args.warmup, 3)):
        eng.align_resident(batch, args.mode)
    if dist:
        dist.barrier()
    ms, cells, launches, nfrag = [], 0, 0, 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            res, t = timed(lambda: eng.align_resident(batch, args.mode))
            st = eng.last_stats()
            ms.append(t)
            cells += cells_of(st)
            launches += st["kernel_launches"]
            nfrag = sum(len(f) for f in res)
            last_stats = st
    dev = "cuda" if dist is not None and dist.get_backend() == "nccl" else "cpu"
    tot_ms = R.max_over_ranks(sum(ms), dist, dev)  # the slowest rank bounds the step
    all_cells = R.sum_over_ranks(cells, dist, dev)
    gcups = all_cells / (tot_ms * 1e-3) / 1e9
    pairs_s = R.whole_job_rate(n * args.steps, world, tot_ms)

    # ---- the seed-scan kernel alone: the lanes of the timed steps run kernels concurrently, so its launch times are
    # taken from single-lane steps (same batch, CUDA events around every scan launch on the context's stream)
    scan_ms, scan_cells, single_ms = 0.0, 0, 0.0
    if rank == 0:
        eng.set_lanes(1, 1)
        for k in range(3):
            res, t = timed(lambda: eng.align_resident(batch, args.mode))
            if k:
                st = eng.last_stats()
                scan_ms += st["ms_scan_kernel"]
                scan_cells += st["cells_scan"]
                single_ms += t
        eng.set_lanes(tuned["lanes"], tuned["bins"])
    eng.free_batch(batch)

    # ---- e2e: host buffers through the public call (H2D, pipeline, D2H of the fragments)
    # (the dcns_pair pointer table over the host sequences is built once, as a C/C++ caller holds it; every timed
    # step copies the sequences to the device and the fragments back)
    e2e_ms, e2e_cells, d2h = [], 0, 0
    prepared = eng.prepare(pairs)
    for _ in range(1):
        eng.align_prepared(prepared, args.mode)
    for _ in range(args.steps):
        res, t = timed(lambda: eng.align_prepared(prepared, args.mode))
        e2e_ms.append(t)
        e2e_cells += cells_of(eng.last_stats())
        h2d_bytes = eng.last_stats()["bytes_h2d"]  # the codes and per-sequence offsets the call copied
        d2h = sum(len(f) for f in res) * (7 * 8 + 16) + sum(len(x.cigar) for f in res for x in f) * 4
    e2e_tot = R.max_over_ranks(sum(e2e_ms), dist, dev)
    e2e_all_cells = R.sum_over_ranks(e2e_cells, dist, dev)

    if rank != 0:
        dist.barrier() if dist else None
        return

    # ---- roofline of the dominant kernel (seed scan)
    peak = eng.measure_scan_roofline()
    achieved = scan_cells / (scan_ms * 1e-3) / 1e9 if scan_ms > 0 else None
    roofline = {"bound": "int-issue", "kernel": "scan_kernel<38>", "achieved": round(achieved, 2) if achieved else None,
                "peak": round(peak, 2), "unit": "GCUPS", "frac": round(achieved / peak, 4) if achieved else None,
                "peak_kind": "measured live: the scan's per-cell int16x2 instruction mix at full occupancy",
                "traffic": round(SCAN_DRAM_BYTES_PER_CELL * level0_cells(pairs) / 1e9, 4) if args.mode == 1 else None,
                "traffic_unit": "GB per level-0 launch (ncu bytes per cell x this batch's level-0 cells)",
                "scan_share_of_single_lane_step": round(scan_ms / single_ms, 4),
                "single_lane_ms_per_step": round(single_ms / 2, 2),
                "timing": "CUDA events around each scan launch, two single-lane steps after the timed region"}

    extras = {}
    if not args.no_extras:
        # one pair per call (the plain per-pair launch form) on a subset
        sub = pairs[:200]
        t0 = time.perf_counter()
        c = 0
        for p in sub:
            eng.align_pairs([p], args.mode)
            c += cells_of(eng.last_stats())
        dt = time.perf_counter() - t0
        extras["per_pair_launch"] = {"value": round(c / dt / 1e9, 4), "unit": "GCUPS", "pairs": len(sub),
                                     "pairs_per_s": round(len(sub) / dt, 2),
                                     "batched_speedup": round(gcups / max(c / dt / 1e9, 1e-12), 2)}
        # continuous batching: Poisson arrivals; a waiter thread records each request's completion as it happens
        def serve(rate, reqs, seed):
            rng = np.random.default_rng(seed)
            eng.serve_start(args.mode, max_inflight=512)
            tick, t_sub, t_done = [], [], [0.0] * len(reqs)

            def waiter():
                for k in range(len(reqs)):
                    while len(tick) <= k:
                        time.sleep(0.0002)
                    eng.wait(tick[k])
                    t_done[k] = time.perf_counter()

            wt = threading.Thread(target=waiter)
            wt.start()
            t_start = t_next = time.perf_counter()
            for a, b in reqs:
                t_next += rng.exponential(1.0 / rate)
                while (gap := t_next - time.perf_counter()) > 0:
                    if gap > 0.001:
                        time.sleep(gap - 0.0005)
                t_sub.append(time.perf_counter())
                tick.append(eng.submit(a, b))
            wt.join()
            t_end = time.perf_counter()
            eng.serve_stop()
            lat_ms = np.array([d - s0 for d, s0 in zip(t_done, t_sub)]) * 1e3
            return {"arrival_rate_per_s": rate, "requests": len(reqs),
                    "pairs_per_s": round(len(reqs) / (t_end - t_start), 2),
                    "p50_ms": round(float(np.percentile(lat_ms, 50)), 2),
                    "p99_ms": round(float(np.percentile(lat_ms, 99)), 2)}

        extras["serving"] = serve(2000.0, pairs[:1500], 3)
        extras["serving_high_rate"] = serve(20000.0, pairs[:4000], 4)
        # the serving workload's own request shapes: a long tail of 50-100 kb requests among short ones
        from dcns_gb300 import workloads as W
        extras["serving_long_tail"] = {
            "workload": "1,200 requests: log-normal median 4 kb, sigma 1.0, 0.2-100 kb, 10 % of 50-100 kb",
            **serve(1000.0, W.serving_requests(n_requests=1200), 5)}

        # the other benchmark configurations, each on its own sample with its own CPU baseline and clock record
        threads = host_threads()
        extras["two_gap"] = line_two_gap(eng, timed, pairs, threads, local)
        extras["long_pairs"] = line_long_pairs(eng, timed, threads, local, peak)
        extras["seeded_chromosome"] = line_seeded_chromosome(eng, timed, threads, local)
        extras["extension_seeds"] = line_extension_seeds(eng, args.ext_seeds, threads, local)

    threads = host_threads()
    sample, desc = cpu_sample(pairs, threads)
    cb = cpu_baseline(sample, desc, args.mode, threads)
    line = {
        "metric": METRIC, "value": round(gcups, 3), "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(tot_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16x2 (seed scan) / int32", "data": "synthetic (seeded)",
        "config": bench_config(n, args.mode, world), "pipeline": tuned,
        "pairs_per_s": round(pairs_s, 2), "fragments": nfrag,
        "e2e": {"value": round(e2e_all_cells / (e2e_tot * 1e-3) / 1e9, 3), "unit": "GCUPS",
                "pairs_per_s": round(R.whole_job_rate(n * args.steps, world, e2e_tot), 2),
                "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h},
        "roofline": roofline, "cpu_baseline": cb, "gpu_launches": launches, "clocks": clk.summary(),
        "stages_ms": {k: round(last_stats[k], 2) for k in ("ms_scan_kernel", "ms_scan_prep", "ms_scan_xfer",
                                                            "ms_replay", "ms_link", "ms_xdrop", "ms_xdrop_kernel",
                                                            "ms_xdrop_tb_kernel", "ms_semiglobal", "ms_total")},
        "rounds": {k: last_stats[k] for k in ("scan_rounds", "xdrop_rounds", "kernel_launches", "seeds",
                                              "xdrop_passes", "tasks_scan")},
    }
    line.update(extras)
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()


if __name__ == "__main__":
    main()
