"""The CUDA path against what the unmodified reference computed on the benchmark workloads themselves
(tests/golden/configs.npz, per-pair digests of fragments and CIGARs made by tests/golden/make_config_golden.py):
the whole 10,000-pair batched workload through both the host-buffer call and a resident batch (four-lane binned
pipeline), its first 500 pairs on the 2-piece path, 10,000 extension-stress seeds, and serving requests through the
continuous-batching loop.  Integer fields and CIGARs bit-exact; p/e sums within 1e-12 relative."""
import numpy as np
import pytest

import config_digest as D
from dcns_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(lib):
    return lib


@pytest.fixture(scope="module")
def c2(configs):
    pairs = W.config2(n_pairs=10000)
    if D.inputs_hash(pairs) != str(configs["c2_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    return pairs


@pytest.fixture(scope="module")
def c5():
    return W.config5(n_requests=2000)


def _assert_digests(got, configs, section, count=None):
    sl = slice(0, count)
    bad, bad_pe = D.compare_pairs(got, configs[section + "_nfrag"][sl], configs[section + "_hash"][sl],
                                  configs[section + "_pe"][sl])
    assert len(bad) == 0, f"{len(bad)} pairs differ from the reference, first {bad[:10].tolist()}"
    assert len(bad_pe) == 0, f"{len(bad_pe)} pairs' p/e-values differ, first {bad_pe[:10].tolist()}"


def test_config2_full_workload_1gap_vs_reference(eng, configs, c2):
    _assert_digests(eng.align_pairs(c2, 1), configs, "c2p1")
    b = eng.upload(c2)
    try:
        _assert_digests(eng.align_resident(b, 1), configs, "c2p1")
    finally:
        eng.free_batch(b)


def test_config2_first500_2gap_vs_reference(eng, configs, c2):
    _assert_digests(eng.align_pairs(c2[:500], 2), configs, "c2p2")


def test_config4_extension_stress_vs_reference(eng, configs):
    tasks = W.config4(n_seeds=10000)
    if D.inputs_hash(tasks) != str(configs["c4_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    out, _ = eng.SemiGlobal_xextend(tasks, cigar=False)
    np.testing.assert_array_equal(out[:, :3], configs["c4_nocigar"])
    out, cigars = eng.SemiGlobal_xextend(tasks, cigar=True)
    np.testing.assert_array_equal(out[:, :5], configs["c4_cigar"])
    hs = np.array([D.cigar_hash(c) for c in cigars], np.uint64)
    bad = np.nonzero(hs != configs["c4_cigar_hash"])[0]
    assert len(bad) == 0, bad[:10].tolist()


def test_config5_serving_requests_vs_reference(eng, configs, c5):
    idx = configs["c5_index"]
    reqs = [c5[i] for i in idx]
    if D.inputs_hash(reqs) != str(configs["c5_inputs"]):
        pytest.skip("the seeded generator drew different inputs on this machine than where the fixture was made")
    eng.serve_start(1, max_inflight=64)
    try:
        tickets = [eng.submit(a, b) for a, b in reqs]
        served = [eng.wait(t) for t in tickets]
    finally:
        eng.serve_stop()
    _assert_digests(served, configs, "c5p1")
    _assert_digests(eng.align_pairs(reqs, 1), configs, "c5p1")


def test_config5_long_requests_same_alone_and_in_mix(eng, c5):
    """The serving workload's long tail (50-100 kb before masking, beyond the reference fixture): each long request
    gives the same fragments alone, in a served mix with short requests, and in one batch call."""
    long = [p for p in c5 if min(len(p[0]), len(p[1])) > 42500][:3]
    short = [p for p in c5 if max(len(p[0]), len(p[1])) < 8000][:30]
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
