"""The oracle restatement against what the unmodified reference computed on the benchmark workloads themselves
(tests/golden/workload_digests.npz): the inputs regenerate bit-identically from their seeded generators, and the oracle
reproduces the reference's digests on a leading sample of every section (the GPU tests compare the CUDA path on the
whole workloads)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import digest as D
from dcns_gb300 import workloads as W


@pytest.fixture(scope="module")
def batch():
    return W.batched_pairs(n_pairs=10000)  # length arrays are drawn up front: a prefix needs the whole workload


@pytest.fixture(scope="module")
def serving():
    return W.serving_requests(n_requests=2000)


def test_workload_inputs_regenerate_identically(ref_digests, batch, serving):
    assert D.inputs_hash(batch) == str(ref_digests["batch_inputs"])
    assert D.inputs_hash(W.extension_seeds(n_seeds=10000)) == str(ref_digests["seeds_inputs"])
    idx = ref_digests["serving_index"]
    assert all(max(len(serving[i][0]), len(serving[i][1])) <= 20000 for i in idx)
    assert D.inputs_hash([serving[i] for i in idx]) == str(ref_digests["serving_inputs"])
    # the serving workload's long tail: about a tenth of the requests above 50 kb before masking (42.5 kb after)
    long = np.mean([max(len(a), len(b)) > 42500 for a, b in serving])
    assert 0.06 < long < 0.14


def _oracle_find(oracle, pairs, two_gap):
    with ThreadPoolExecutor(max_workers=8) as ex:
        return list(ex.map(lambda ab: oracle.find(ab[0], ab[1], two_gap=two_gap)[0], pairs))


@pytest.mark.parametrize("section,two_gap,count", [("batch_1gap", False, 48), ("batch_2gap", True, 16), ("serving_1gap", False, 24)])
def test_oracle_matches_reference_digests(oracle, ref_digests, batch, serving, section, two_gap, count):
    if section == "serving_1gap":
        pairs = [serving[i] for i in ref_digests["serving_index"][:count]]
    else:
        pairs = batch[:count]
    bad, bad_pe = D.compare_pairs(_oracle_find(oracle, pairs, two_gap), ref_digests[section + "_nfrag"][:count],
                                  ref_digests[section + "_hash"][:count], ref_digests[section + "_pe"][:count])
    assert len(bad) == 0 and len(bad_pe) == 0, (bad[:10], bad_pe[:10])


def test_oracle_matches_reference_extension_stress(oracle, ref_digests):
    tasks = W.extension_seeds(n_seeds=2000)  # drawn seed by seed: the first 2,000 of the 10,000-seed workload
    for k, (a, b) in enumerate(tasks):
        e = oracle.xextend(a, b)
        assert (e["score"], e["end1"], e["end2"]) == tuple(int(v) for v in ref_digests["seeds_nocigar"][k]), k
        e = oracle.xextend(a, b, cigar=True)
        assert (e["score"], e["end1"], e["end2"], e["iii"], e["jjj"]) == tuple(int(v) for v in ref_digests["seeds_cigar"][k]), k
        assert D.cigar_hash(e["cigar"]) == int(ref_digests["seeds_cigar_hash"][k]), k
