"""The CUDA path against what the unmodified reference computed on the benchmark workloads themselves
(tests/golden/workload_digests.npz, per-pair digests of fragments and CIGARs made by
tests/golden/make_workload_digests.py): the whole 10,000-pair batched workload through both the host-buffer call and a
resident batch (four-lane binned pipeline), its first 500 pairs on the 2-piece path, 10,000 extension-stress seeds, and
serving requests through the continuous-batching loop.  The long shapes (tests/golden/long_digests.npz and
seeded_chromosome.npz, made by the reference with a lazily stored traceback matrix, and by the oracle where it says
so): four whole 200 kb long pairs, the serving workload's 50-100 kb requests, and cut2Gaps2's seeded overload on a whole
200 kb pair without a length cap.  Integer fields and CIGARs bit-exact; p/e sums within 1e-12 relative."""
import numpy as np
import pytest

import digest as D
from dcns_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(lib):
    return lib


@pytest.fixture(scope="module")
def batch(ref_digests):
    pairs = W.batched_pairs(n_pairs=10000)
    if D.inputs_hash(pairs) != str(ref_digests["batch_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    return pairs


@pytest.fixture(scope="module")
def serving():
    return W.serving_requests(n_requests=2000)


@pytest.fixture(scope="module")
def long_digests():
    import os
    from conftest import GOLDEN_DIR
    return np.load(os.path.join(GOLDEN_DIR, "long_digests.npz"))


def _assert_digests(got, ref_digests, section, count=None):
    sl = slice(0, count)
    bad, bad_pe = D.compare_pairs(got, ref_digests[section + "_nfrag"][sl], ref_digests[section + "_hash"][sl],
                                  ref_digests[section + "_pe"][sl])
    assert len(bad) == 0, f"{len(bad)} pairs differ from the reference, first {bad[:10].tolist()}"
    assert len(bad_pe) == 0, f"{len(bad_pe)} pairs' p/e-values differ, first {bad_pe[:10].tolist()}"


def test_batched_pairs_full_workload_1gap_vs_reference(eng, ref_digests, batch):
    _assert_digests(eng.align_pairs(batch, 1), ref_digests, "batch_1gap")
    b = eng.upload(batch)
    try:
        _assert_digests(eng.align_resident(b, 1), ref_digests, "batch_1gap")
    finally:
        eng.free_batch(b)


def test_batched_pairs_first500_2gap_vs_reference(eng, ref_digests, batch):
    _assert_digests(eng.align_pairs(batch[:500], 2), ref_digests, "batch_2gap")


def test_extension_seeds_vs_reference(eng, ref_digests):
    tasks = W.extension_seeds(n_seeds=10000)
    if D.inputs_hash(tasks) != str(ref_digests["seeds_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    out, _ = eng.SemiGlobal_xextend(tasks, cigar=False)
    np.testing.assert_array_equal(out[:, :3], ref_digests["seeds_nocigar"])
    out, cigars = eng.SemiGlobal_xextend(tasks, cigar=True)
    np.testing.assert_array_equal(out[:, :5], ref_digests["seeds_cigar"])
    hs = np.array([D.cigar_hash(c) for c in cigars], np.uint64)
    bad = np.nonzero(hs != ref_digests["seeds_cigar_hash"])[0]
    assert len(bad) == 0, bad[:10].tolist()


def test_serving_requests_vs_reference(eng, ref_digests, serving):
    idx = ref_digests["serving_index"]
    reqs = [serving[i] for i in idx]
    if D.inputs_hash(reqs) != str(ref_digests["serving_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    eng.serve_start(1, max_inflight=64)
    try:
        tickets = [eng.submit(a, b) for a, b in reqs]
        served = [eng.wait(t) for t in tickets]
    finally:
        eng.serve_stop()
    _assert_digests(served, ref_digests, "serving_1gap")
    _assert_digests(eng.align_pairs(reqs, 1), ref_digests, "serving_1gap")


def test_serving_long_requests_same_alone_and_in_mix(eng, serving):
    """The serving workload's long tail (50-100 kb before masking, beyond the reference fixture): each long request
    gives the same fragments alone, in a served mix with short requests, and in one batch call."""
    long = [p for p in serving if min(len(p[0]), len(p[1])) > 42500][:3]
    short = [p for p in serving if max(len(p[0]), len(p[1])) < 8000][:30]
    assert len(long) == 3
    mix = short[:10] + long[:1] + short[10:20] + long[1:] + short[20:]
    alone = [eng.align_pairs([p], 1)[0] for p in long]
    eng.serve_start(1, max_inflight=16)
    try:
        tickets = [eng.submit(a, b) for a, b in mix]
        served = [eng.wait(t) for t in tickets]
    finally:
        eng.serve_stop()
    batch = eng.align_pairs(mix, 1)
    pos = [10, 21, 22]
    for k, i in enumerate(pos):
        assert D.fragments_hash(served[i]) == D.fragments_hash(alone[k]) == D.fragments_hash(batch[i]), k
    for i in range(len(mix)):
        assert D.fragments_hash(served[i]) == D.fragments_hash(batch[i]), i


def test_long_pairs_200kb_full_size_vs_reference(eng, long_digests):
    """Four whole 200 kb x ~234 kb pairs of the long-pair workload (row-chunked seed scan with warm-ups, wide x-drop
    bands) against the reference's own fragments of the same pairs (also computed by the oracle, which agreed)."""
    pairs = W.long_pairs_200kb(n_pairs=4)
    if D.inputs_hash(pairs) != str(long_digests["long_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    _assert_digests(eng.align_pairs(pairs, 1), long_digests, "long_1gap")


def test_serving_long_tail_vs_reference(eng, long_digests, serving):
    """The serving workload's 50-100 kb class (20 requests) served through the loop between short requests, and in
    one batch call, against the reference's fragments."""
    idx = long_digests["serving_long_index"]
    reqs = [serving[i] for i in idx]
    if D.inputs_hash(reqs) != str(long_digests["serving_long_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    short = [p for p in serving if max(len(p[0]), len(p[1])) < 8000][:40]
    mix = [x for k, r in enumerate(reqs) for x in (r, short[2 * k], short[2 * k + 1])]
    eng.serve_start(1, max_inflight=16)
    try:
        tickets = [eng.submit(a, b) for a, b in mix]
        served = [eng.wait(t) for t in tickets]
    finally:
        eng.serve_stop()
    _assert_digests(served[0::3], long_digests, "serving_long_1gap")
    _assert_digests(eng.align_pairs(reqs, 1), long_digests, "serving_long_1gap")


def test_seeded_two_gap_whole_200kb_pair_no_cap_vs_reference(eng):
    """cut2Gaps2's seeded overload on a whole 200 kb x ~234 kb pair with no length cap (max_align_len 0): past the
    140 kb the reference's driver caps it at, whose dense traceback matrix would be 40 GB here; the engine keeps
    banded direction codes.  Against the reference's fragments (lazily stored matrix) and the oracle's, which agreed."""
    import os
    from conftest import GOLDEN_DIR
    z = np.load(os.path.join(GOLDEN_DIR, "seeded_chromosome.npz"))
    a, b = W.long_pairs_200kb(n_pairs=1)[0]
    if D.inputs_hash([(a, b)]) != str(z["inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    seeds = [tuple(int(v) for v in s) for s in z["seeds"]]
    got = eng.align_seeded([(a, b)], [seeds], max_align_len=0)[0]
    exp = [(tuple(int(v) for v in z["frag"][k]), [int(c) for c in z["cigar"][z["cigar_off"][k]:z["cigar_off"][k + 1]]])
           for k in range(len(z["frag"]))]
    assert [(f.start1, f.end1, f.start2, f.end2, f.score) for f in got] == [e[0] for e in exp]
    assert [list(f.cigar) for f in got] == [e[1] for e in exp]
    for f, pe in zip(got, z["pe"]):
        assert f.pvalue == pytest.approx(float(pe[0]), rel=1e-12, abs=0)
