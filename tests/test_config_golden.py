"""The oracle restatement against what the unmodified reference computed on the benchmark workloads themselves
(tests/golden/configs.npz): the inputs regenerate bit-identically from their seeded generators, and the oracle
reproduces the reference's digests on a leading sample of every section (the GPU tests compare the CUDA path on the
whole workloads)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import config_digest as D
from dcns_gb300 import workloads as W


@pytest.fixture(scope="module")
def c2():
    return W.config2(n_pairs=10000)  # length arrays are drawn up front: a prefix needs the whole workload


@pytest.fixture(scope="module")
def c5():
    return W.config5(n_requests=2000)


def test_config_inputs_regenerate_identically(configs, c2, c5):
    assert D.inputs_hash(c2) == str(configs["c2_inputs"])
    assert D.inputs_hash(W.config4(n_seeds=10000)) == str(configs["c4_inputs"])
    reqs = c5
    idx = configs["c5_index"]
    assert all(max(len(reqs[i][0]), len(reqs[i][1])) <= 20000 for i in idx)
    assert D.inputs_hash([reqs[i] for i in idx]) == str(configs["c5_inputs"])
    # the serving workload's long tail: about a tenth of the requests above 50 kb before masking (42.5 kb after)
    long = np.mean([max(len(a), len(b)) > 42500 for a, b in reqs])
    assert 0.06 < long < 0.14


def _oracle_find(oracle, pairs, two_gap):
    with ThreadPoolExecutor(max_workers=8) as ex:
        return list(ex.map(lambda ab: oracle.find(ab[0], ab[1], two_gap=two_gap)[0], pairs))


@pytest.mark.parametrize("section,two_gap,count", [("c2p1", False, 48), ("c2p2", True, 16), ("c5p1", False, 24)])
def test_oracle_matches_reference_digests(oracle, configs, c2, c5, section, two_gap, count):
    if section == "c5p1":
        pairs = [c5[i] for i in configs["c5_index"][:count]]
    else:
        pairs = c2[:count]
    bad, bad_pe = D.compare_pairs(_oracle_find(oracle, pairs, two_gap), configs[section + "_nfrag"][:count],
                                  configs[section + "_hash"][:count], configs[section + "_pe"][:count])
    assert len(bad) == 0 and len(bad_pe) == 0, (bad[:10], bad_pe[:10])


def test_oracle_matches_reference_extension_stress(oracle, configs):
    tasks = W.config4(n_seeds=2000)  # drawn seed by seed: the first 2,000 of the 10,000-seed workload
    for k, (a, b) in enumerate(tasks):
        e = oracle.xextend(a, b)
        assert (e["score"], e["end1"], e["end2"]) == tuple(int(v) for v in configs["c4_nocigar"][k]), k
        e = oracle.xextend(a, b, cigar=True)
        assert (e["score"], e["end1"], e["end2"], e["iii"], e["jjj"]) == tuple(int(v) for v in configs["c4_cigar"][k]), k
        assert D.cigar_hash(e["cigar"]) == int(configs["c4_cigar_hash"][k]), k
