"""Parity of the CUDA path with the reference: golden fixtures (generated by the unmodified reference) and the oracle
restatement on fresh seeded inputs.  Integer fields (scores, coordinates, CIGARs, seed sets) must be bit-exact;
p/e-values are FP64 from identical scores and must agree to 1e-12 relative (libm exp may differ by an ulp)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from conftest import ragged
from dcns_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL = 1e-12


@pytest.fixture(scope="module")
def eng(lib):
    return lib


def frag_keys(frs):
    return [f.key() for f in frs]


def assert_same_fragments(got, exp, ctx=""):
    assert frag_keys(got) == frag_keys(exp), ctx
    for g, e in zip(got, exp):
        assert g.pvalue == pytest.approx(e.pvalue, rel=REL, abs=0), ctx
        assert g.evalue == pytest.approx(e.evalue, rel=REL, abs=0), ctx


# ------------------------------------------------------------------ kernel level vs golden
def test_smith_waterman_golden(eng, golden):
    z = golden
    n = len(z["sw_exp"])
    groups = {}
    for i in range(n):
        groups.setdefault(tuple(int(v) for v in z["sw_prm"][i]), []).append(i)
    for (o, e, m, x), ids in groups.items():
        tasks = [(ragged(z, "sw_a", i), ragged(z, "sw_b", i)) for i in ids]
        out = eng.SmithWaterman(tasks, open1=o, ext1=e, match=m, mismatch=x)
        for k, i in enumerate(ids):
            exp = tuple(int(v) for v in z["sw_exp"][i])
            assert int(out[k, 0]) == exp[0], i
            if exp[0] > 0 and exp[1] != -7:
                assert tuple(int(v) for v in out[k]) == exp, i


def test_known_answer_inline_sequences(eng, golden):
    z = golden
    tasks = [(ragged(z, "ka_a", i), ragged(z, "ka_b", i)) for i in range(len(z["ka_sw"]))]
    sw = eng.SmithWaterman(tasks)
    xe, xc = eng.SemiGlobal_xextend(tasks, cigar=True)
    sg, sc = eng.SemiGlobal(tasks, cigar=True, open2=-80, ext2=-1, zdrop=100, bandwidth=100)
    for i in range(len(tasks)):
        assert int(sw[i, 0]) == int(z["ka_sw"][i, 0])
        assert tuple(int(v) for v in xe[i, :5]) == tuple(int(v) for v in z["ka_xe"][i])
        assert xc[i] == [int(c) for c in ragged(z, "ka_cigar", 2 * i)]
        assert tuple(int(v) for v in sg[i, :3]) == tuple(int(v) for v in z["ka_sg"][i])
        assert sc[i] == [int(c) for c in ragged(z, "ka_cigar", 2 * i + 1)]


def test_smith_waterman_long_tasks_vs_oracle(eng, oracle):
    """Large kernel-level SmithWaterman calls, which the engine runs as one-warp wavefronts: both sequences too long
    for the reference's striped kernels (its scalar semantics, impl/sequenceAlignment3.cpp:223-225) and long pairs
    the striped int16 kernel still takes, against the oracle's own dispatch, with N runs, planted similarity, a task
    whose maximum sits in the last rows and a non-default scoring."""
    rng = np.random.default_rng(17000)
    tasks = []
    for n1, n2 in [(21000, 20000), (17000, 16500), (12000, 30000)]:
        a, b = W.planted_pair(rng, n1, n2, 6, 100, 900, 0.8, 0.95, 0.01, 0.1)
        tasks.append((W.prepare(a), W.prepare(b)))
    a, b = tasks[0]
    tasks[0] = (np.concatenate([a, b[-3000:]]), b)  # a copy of the read's tail at the reference's end
    for kw in ({}, {"open1": -5, "ext1": -1, "match": 3, "mismatch": -4}):
        out = eng.SmithWaterman(tasks, **kw)
        okw = {"open": kw.get("open1", -4), "ext": kw.get("ext1", -2), "match": kw.get("match", 2),
               "mismatch": kw.get("mismatch", -3)}
        for k, (a, b) in enumerate(tasks):
            assert tuple(int(v) for v in out[k]) == oracle.sw(a, b, mode=0, **okw), (k, kw)


def test_xextend_golden(eng, golden):
    z = golden
    n = len(z["xe_exp"])
    groups = {}
    for i in range(n):
        groups.setdefault(tuple(int(v) for v in z["xe_prm"][i]), []).append(i)
    for (w, xd, cig), ids in groups.items():
        tasks = [(ragged(z, "xe_a", i), ragged(z, "xe_b", i)) for i in ids]
        out, cigars = eng.SemiGlobal_xextend(tasks, cigar=bool(cig), w=w, xdrop=xd)
        for k, i in enumerate(ids):
            assert tuple(int(v) for v in out[k, :5]) == tuple(int(v) for v in z["xe_exp"][i]), i
            assert cigars[k] == [int(c) for c in ragged(z, "xe_cigar", i)], i


def test_semiglobal_golden(eng, golden):
    z = golden
    n = len(z["sg_exp"])
    groups = {}
    for i in range(n):
        groups.setdefault(tuple(int(v) for v in z["sg_prm"][i]), []).append(i)
    for (bw, zd, o2, e2, cig), ids in groups.items():
        tasks = [(ragged(z, "sg_a", i), ragged(z, "sg_b", i)) for i in ids]
        out, cigars = eng.SemiGlobal(tasks, cigar=bool(cig), bandwidth=bw, zdrop=zd, open2=o2, ext2=e2)
        for k, i in enumerate(ids):
            assert tuple(int(v) for v in out[k, :3]) == tuple(int(v) for v in z["sg_exp"][i]), (i, bw, zd, o2, e2)
            assert cigars[k] == [int(c) for c in ragged(z, "sg_cigar", i)], i


def test_sliding_window_golden(eng, golden):
    z = golden
    seqs = [ragged(z, "sl_seq", i) for i in range(len(z["sl_seq_off"]) - 1)]
    rows = {(int(j), int(i)): str(t) for (j, i), t in zip(z["sl_rows"], z["sl_text"])}
    sc, _ = eng.slidingWindowAlignment(seqs)
    for i in range(1, len(seqs)):
        for k in range(sc.shape[1]):
            assert "%g" % sc[i - 1, k] == rows[(k * 8, i)], (i, k)


# ------------------------------------------------------------------ whole path vs golden
def _golden_fragments(z, name):
    from oracle.oracle import Fragment
    out, k = [], 0
    for n in z[name + "_nfrag"]:
        fr = []
        for _ in range(int(n)):
            f = [int(v) for v in z[name + "_frag"][k]]
            pe = z[name + "_pe"][k]
            fr.append(Fragment(*f, [int(c) for c in ragged(z, name + "_cigar", k)], float(pe[0]), float(pe[1])))
            k += 1
        out.append(fr)
    return out


@pytest.mark.parametrize("name,mode", [("p1", 1), ("p2", 2)])
def test_pipeline_golden_batched(eng, golden, name, mode):
    z = golden
    pairs = [(ragged(z, "pp_a", i), ragged(z, "pp_b", i)) for i in range(len(z["pp_a_off"]) - 1)]
    exp = _golden_fragments(z, name)
    got = eng.align_pairs(pairs, mode)
    for i in range(len(pairs)):
        assert_same_fragments(got[i], exp[i], (name, i))


@pytest.mark.parametrize("mode", [1, 2])
def test_pipeline_golden_per_pair(eng, golden, mode):
    """Single-pair calls take the row-chunked scan path (few tiles); results must not change."""
    z = golden
    name = "p1" if mode == 1 else "p2"
    exp = _golden_fragments(z, name)
    for i in (0, 3, 7):
        a, b = ragged(z, "pp_a", i), ragged(z, "pp_b", i)
        got = eng.align_pairs([(a, b)], mode)[0]
        assert_same_fragments(got, exp[i], (name, i))


# ------------------------------------------------------------------ fresh inputs vs the oracle
def _oracle_many(oracle, pairs, two_gap):
    with ThreadPoolExecutor(max_workers=8) as ex:
        return list(ex.map(lambda ab: oracle.find(ab[0], ab[1], two_gap=two_gap)[0], pairs))


def test_batched_pairs_sample_vs_oracle(eng, oracle):
    pairs = W.batched_pairs(n_pairs=96, seed=4242)
    exp = _oracle_many(oracle, pairs, False)
    got = eng.align_pairs(pairs, 1)
    for i in range(len(pairs)):
        assert_same_fragments(got[i], exp[i], i)
    st = eng.last_stats()
    assert st["cells_scan"] > 0 and st["seeds"] > 0


def test_two_gap_sample_vs_oracle(eng, oracle):
    pairs = W.batched_pairs(n_pairs=24, seed=777)
    pairs = [(a[:2500], b[:2500]) for a, b in pairs if len(b) >= 8]
    exp = _oracle_many(oracle, pairs, True)
    got = eng.align_pairs(pairs, 2)
    for i in range(len(pairs)):
        assert_same_fragments(got[i], exp[i], i)


def test_seed_scan_random_with_n_and_widths(eng, oracle):
    rng = np.random.default_rng(11)
    for alphabet in (2, 4, 5):
        tasks = [W.random_pair(rng, int(rng.integers(0, 3000)), int(rng.integers(0, 80)), alphabet)
                 for _ in range(300)]
        out = eng.SmithWaterman(tasks)
        for k, (a, b) in enumerate(tasks):
            exp = oracle.sw(a, b)
            assert int(out[k, 0]) == exp[0], k
            if exp[0] > 0:
                assert tuple(int(v) for v in out[k]) == exp, (k, len(a), len(b))


def test_seed_scan_chunking_exact_on_long_gappy_alignments(eng, oracle):
    """Long references with many planted, gapped copies of the same window: maxima that tie across chunk borders
    and alignments that straddle them must resolve exactly as a single sequential scan."""
    rng = np.random.default_rng(5)
    read = rng.integers(0, 4, 38).astype(np.int8)
    read[read >= 2] += 1
    ref = rng.integers(0, 4, 60000).astype(np.int8)
    ref[ref >= 2] += 1
    for pos in range(500, 59000, 1237):
        seg = read.copy()
        if pos % 3 == 0:
            seg = np.concatenate([seg[:19], rng.integers(0, 5, 3).astype(np.int8), seg[19:]])
        ref[pos:pos + len(seg)] = seg
    out = eng.SmithWaterman([(ref, read)])
    assert tuple(int(v) for v in out[0]) == oracle.sw(ref, read)


def test_empty_and_tiny_inputs(eng, oracle):
    rng = np.random.default_rng(3)
    pairs = [(np.zeros(0, np.int8), rng.integers(0, 5, 50).astype(np.int8)),
             (rng.integers(0, 5, 50).astype(np.int8), np.zeros(0, np.int8)),
             (rng.integers(0, 5, 7).astype(np.int8), rng.integers(0, 5, 5).astype(np.int8)),
             (np.full(200, 2, np.int8), np.full(200, 2, np.int8))]
    got = eng.align_pairs(pairs, 1)
    for i, (a, b) in enumerate(pairs):
        assert_same_fragments(got[i], oracle.find(a, b)[0], i)


def test_invalid_codes_rejected(eng):
    import dcns_gb300
    bad = np.array([0, 1, 7, 3], np.int8)
    with pytest.raises(dcns_gb300.DcnsError) as e:
        eng.align_pairs([(bad, bad)], 1)
    assert e.value.code == -1
    # the context stays usable and exact after the rejected call
    a = np.array([0, 1, 3, 4] * 30, np.int8)
    assert eng.SmithWaterman([(a, a[:38])])[0, 0] == 76


def test_non_default_scoring(eng, oracle):
    rng = np.random.default_rng(21)
    x, y = W.planted_pair(rng, 2000, 1800, 8, 40, 200, 0.8, 0.95, 0.01, 0.0)
    a, b = W.prepare(x), W.prepare(y)
    for kw in (dict(match=3, mismatch=-2, open1=-5, ext1=-1, min_score=50),
               dict(match=1, mismatch=-1, open1=-2, ext1=-1, min_score=20, window=30, step=5),
               dict(w=5, xdrop=30)):
        got = eng.findSimilarFragmentsForPairedSequence(a, b, **kw)
        exp, _ = oracle.find(a, b, **kw)
        assert_same_fragments(got, exp, kw)


def test_serving_same_alone_and_in_mix(eng):
    """Continuous batching: each request's result is identical whether it runs alone or mixed with others."""
    pairs = W.batched_pairs(n_pairs=40, seed=99)
    alone = [eng.align_pairs([p], 1)[0] for p in pairs[:6]]
    eng.serve_start(1, max_inflight=16)
    try:
        tickets = [eng.submit(a, b) for a, b in pairs]
        res = [eng.wait(t) for t in tickets]
    finally:
        eng.serve_stop()
    for i in range(6):
        assert frag_keys(res[i]) == frag_keys(alone[i]), i
    batch = eng.align_pairs(pairs, 1)
    for i in range(len(pairs)):
        assert frag_keys(res[i]) == frag_keys(batch[i]), i


def test_resident_batch_matches_host_path(eng):
    pairs = W.batched_pairs(n_pairs=64, seed=31)
    b = eng.upload(pairs)
    try:
        r1 = eng.align_resident(b, 1)
        r2 = eng.align_resident(b, 1)  # the batch stays resident and reusable
    finally:
        eng.free_batch(b)
    ref = eng.align_pairs(pairs, 1)
    for i in range(len(pairs)):
        assert frag_keys(r1[i]) == frag_keys(ref[i]) == frag_keys(r2[i]), i


def test_scan_roofline_probe_positive(eng):
    g = eng.measure_scan_roofline()
    assert 100.0 < g < 1e6


def test_semiglobal_multiwarp_vs_oracle(eng, oracle):
    """Long DPs (many 32-row stripes across the CTA's warps, FIFO wrap-around), narrow bands, empty-band tails
    (rows past n2 + w) and early z-drop stops, with and without CIGAR."""
    rng = np.random.default_rng(17)
    cases = []
    for n1, n2 in ((3000, 2000), (700, 4000), (5000, 300), (257, 257), (33, 1000), (1, 5)):
        x, y = W.planted_pair(rng, n1, n2, 3, 40, 200, 0.8, 0.95, 0.01, 0.0)
        cases.append((W.prepare(x), W.prepare(y)))
    for bw, zd, o2, e2 in ((20000, 50, -45, 0), (100, 50, -45, 0), (7, 30, -20, -1), (300, 10, -80, -1)):
        for cig in (False, True):
            out, cigars = eng.SemiGlobal(cases, cigar=cig, bandwidth=bw, zdrop=zd, open2=o2, ext2=e2)
            for k, (a, b) in enumerate(cases):
                exp = oracle.semiglobal(a, b, cigar=cig, bandwidth=bw, zdrop=zd, open2=o2, ext2=e2)
                assert tuple(int(v) for v in out[k, :3]) == (exp["score"], exp["end1"], exp["end2"]), (k, bw, zd)
                assert cigars[k] == exp["cigar"], (k, bw, zd, cig)


def test_binned_two_lane_batch_vs_oracle(eng, oracle):
    # 4200 pairs take the path that splits a batch into bins run on two lanes (batches of at least 4096 pairs)
    rng = np.random.default_rng(4096)
    pairs = []
    for _ in range(4200):
        a, b = W.planted_pair(rng, int(rng.integers(150, 700)), int(rng.integers(150, 700)), int(rng.integers(0, 4)),
                              30, 120, 0.7, 0.95, 0.01, 0.1)
        pairs.append((W.prepare(a), W.prepare(b)))
    exp = _oracle_many(oracle, pairs, False)
    got = eng.align_pairs(pairs, 1)
    assert len(got) == len(pairs)
    for i in range(len(pairs)):
        assert_same_fragments(got[i], exp[i], i)


@pytest.mark.parametrize("cigar", [False, True])
def test_xdrop_stress_extension_seeds_vs_oracle(eng, oracle, cigar):
    """Extension-stress seeds (flanks 50-2000 bp, identity 50-98 %, indels 0-3 %): band restarts up to wide bands,
    reverse passes longer than the first traceback slot, variable termination."""
    tasks = W.extension_seeds(3000, seed=44)
    out, cigars = eng.SemiGlobal_xextend(tasks, cigar=cigar)
    for k, (a, b) in enumerate(tasks):
        e = oracle.xextend(a, b, cigar=cigar)
        assert tuple(int(v) for v in out[k, :5]) == (e["score"], e["end1"], e["end2"], e["iii"], e["jjj"]), k
        if cigar:
            assert cigars[k] == e["cigar"], k


def test_long_pairs_200kb_subsets_vs_oracle(eng, oracle):
    """Long-pair shapes of the 200 kb workload at sizes the oracle finishes quickly: a 200 kb reference against a 4 kb
    query slice and a 4 kb reference slice against the 200 kb query (row chunking with warm-ups, many windows)."""
    a, b = W.long_pairs_200kb(n_pairs=1)[0]
    pairs = [(a, b[100000:104000]), (a[50000:54000], b), (a[:30000], b[:30000])]
    exp = _oracle_many(oracle, pairs, False)
    got = eng.align_pairs(pairs, 1)
    for i in range(len(pairs)):
        assert_same_fragments(got[i], exp[i], i)


def test_long_pairs_200kb_full_size_alone_equals_in_batch(eng):
    """At full size (200 kb x 234 kb) the fragments of a pair do not depend on how its scan is tiled: alone (few
    tiles, rows split into chunks with warm-ups) and inside a batch of other pairs (different chunking)."""
    a, b = W.long_pairs_200kb(n_pairs=1)[0]
    alone = eng.align_pairs([(a, b)], 1)[0]
    others = W.batched_pairs(n_pairs=300, seed=31)
    mixed = eng.align_pairs(others[:150] + [(a, b)] + others[150:], 1)[150]
    assert len(alone) > 50
    assert frag_keys(alone) == frag_keys(mixed)
    assert [f.cigar for f in alone] == [f.cigar for f in mixed]


def test_one_reference_many_queries_shared_upload(eng, oracle):
    """The multi-species pattern (one reference x N queries, p-value filter off as that caller sets it,
    getCnsForMultipleSpecies.cpp:126-135): one batched call with the reference packed once gives the oracle's
    per-pair results."""
    rng = np.random.default_rng(515)
    ref_txt = W.planted_pair(rng, 6000, 10, 0, 30, 60, 0.9, 0.9, 0.0, 0.1)[0]
    ref = W.prepare(ref_txt)
    queries = []
    for k in range(40):  # species: diverged copies of (part of) the reference
        lo = int(rng.integers(0, 3000))
        seg = W.mutate(rng, ref_txt[lo:lo + int(rng.integers(1500, 3000))].encode(), float(rng.uniform(0.7, 0.95)),
                       0.01)
        queries.append(W.prepare(seg.decode()))
    got = eng.align_one_to_many(ref, queries, pvalue=1.0)
    for k, q in enumerate(queries):
        assert_same_fragments(got[k], oracle.find(ref, q, pvalue=1.0)[0], k)


@pytest.mark.parametrize("max_align", [0, 400])
def test_seeded_two_gap_vs_oracle(eng, oracle, max_align):
    """cut2Gaps2's seeded overload: reverse DPs of every seed and forward DPs of every distinct start on the device,
    the reference's order, skip test and dedupe replayed on the host."""
    from test_oracle_pin import _seeded_cases

    cases = _seeded_cases(oracle, n=4, seed=7)
    got = eng.align_seeded([(A, B) for A, B, _ in cases], [s for _, _, s in cases], max_align_len=max_align)
    for k, (A, B, seeds) in enumerate(cases):
        exp = oracle.find_seeded(A, B, seeds, max_align if max_align > 0 else 1 << 30)
        assert_same_fragments(got[k], exp, k)


@pytest.mark.parametrize("kw", [dict(), dict(bandwidth=40, zdrop=20, open2=-30, ext2=-1)])
def test_xseed_overload_vs_oracle(eng, oracle, kw):
    """The x-seed overload without maximumAlignLength (the 2-gap overload's 2-piece stage) on caller-given seeds."""
    from test_oracle_pin import _seeded_cases

    cases = _seeded_cases(oracle, n=4, seed=9)
    got = eng.align_xseeds([(A, B) for A, B, _ in cases], [s for _, _, s in cases], **kw)
    for k, (A, B, seeds) in enumerate(cases):
        assert_same_fragments(got[k], oracle.find_xseeds(A, B, seeds, **kw), k)


@pytest.mark.parametrize("pieces,bandwidth", [(1, 20000), (2, 20000), (2, 30), (1, 30)])
def test_weighted_drivers_vs_oracle(eng, oracle, pieces, bandwidth):
    """weighted1Gap / weighted2Gaps: per-row categories (substitution, gap models, z-drop), one warp per DP."""
    from test_oracle_pin import WEIGHT_CATS, _weighted_cases

    cases = _weighted_cases(n=5, seed=11)
    got = eng.align_weighted([(A, B) for A, B, _ in cases], [w for _, _, w in cases], WEIGHT_CATS, pieces,
                             bandwidth=bandwidth)
    for k, (A, B, wts) in enumerate(cases):
        exp = oracle.find_weighted(A, B, wts, WEIGHT_CATS, pieces, bandwidth=bandwidth)
        assert_same_fragments(got[k], exp, k)
