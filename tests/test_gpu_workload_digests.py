"""The CUDA path against what the unmodified reference computed on the benchmark workloads themselves
(tests/golden/workload_digests.npz, per-pair digests of fragments and CIGARs made by
tests/golden/make_workload_digests.py): the whole 10,000-pair batched workload through both the host-buffer call and a resident batch (four-lane binned
pipeline), its first 500 pairs on the 2-piece path, 10,000 extension-stress seeds, and serving requests through the
continuous-batching loop.  Integer fields and CIGARs bit-exact; p/e sums within 1e-12 relative."""
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
