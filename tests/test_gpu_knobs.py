"""Kernel-shape settings never change a result.  Each setting (an environment variable read when a context is
created: the forms the autotuner chooses among) aligns samples of the batched workload, 1-gap and 2-gap, and its
fragments, CIGARs and p/e-values equal those of a context with the default shapes (which the workload-digest tests
pin to the reference's outputs).  The bin settings run a batch large enough to be split into bins."""
import os

import numpy as np
import pytest

import dcns_gb300 as D
from dcns_gb300 import workloads as W

pytestmark = pytest.mark.gpu

KERNEL_KNOBS = [
    {"DCNS_XDROP_RESUME_LANES": "4"},
    {"DCNS_XDROP_RESUME_LANES": "16"},
    {"DCNS_XDROP_RESUME_LANES": "32"},
    {"DCNS_XDROP_HANDOFF": "0"},
    {"DCNS_XDROP_HANDOFF": "48"},
    {"DCNS_XDROP_FLAT": "0"},
    {"DCNS_XDROP_WARP_FROM": "10"},
    {"DCNS_XDROP_WAVE": "0"},
    {"DCNS_SG_FLOW": "0"},
    {"DCNS_SG_FLOW_BLOCKS": "6"},
    {"DCNS_SCAN_TILES": "16"},
    {"DCNS_XDROP_GROUP_FROM": "20"},
    {"DCNS_XDROP_GROUP_FROM": "10"},
    {"DCNS_XDROP_GROUP_FROM": "10", "DCNS_XDROP_RESUME_LANES": "4"},
    {"DCNS_XDROP_GROUP_FROM": "20", "DCNS_XDROP_RESUME_LANES": "16"},
]
BIN_KNOBS = [
    {"DCNS_BINS_BY_SIZE": "1", "DCNS_BIN_RATIO": "1.6"},
    {"DCNS_BINS_BY_SIZE": "1", "DCNS_BIN_RATIO": "0.6", "DCNS_LANES": "3", "DCNS_BINS": "5"},
]


def engine_with(env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return D.Engine(0)
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def flat(results):
    return [[(f.key(), f.pvalue, f.evalue) for f in frs] for frs in results]


@pytest.fixture(scope="module")
def sample():
    return W.batched_pairs(n_pairs=10000)[:600]


@pytest.fixture(scope="module")
def short_pairs():
    rng = np.random.default_rng(4097)
    pairs = []
    for _ in range(4300):
        a, b = W.planted_pair(rng, int(rng.integers(150, 900)), int(rng.integers(150, 900)), int(rng.integers(0, 4)),
                              30, 120, 0.7, 0.95, 0.01, 0.1)
        pairs.append((W.prepare(a), W.prepare(b)))
    return pairs


@pytest.fixture(scope="module")
def defaults(sample, short_pairs):
    e = engine_with({})
    out = {"one": flat(e.align_pairs(sample, 1)), "two": flat(e.align_pairs(sample[:200], 2)),
           "binned": flat(e.align_pairs(short_pairs, 1))}
    e.close()
    return out


@pytest.mark.parametrize("env", KERNEL_KNOBS, ids=lambda e: ",".join(f"{k}={v}" for k, v in e.items()))
def test_kernel_shape_settings_give_the_default_results(env, sample, defaults):
    e = engine_with(env)
    try:
        assert flat(e.align_pairs(sample, 1)) == defaults["one"]
        assert flat(e.align_pairs(sample[:200], 2)) == defaults["two"]
    finally:
        e.close()


@pytest.mark.parametrize("env", BIN_KNOBS, ids=lambda e: ",".join(f"{k}={v}" for k, v in e.items()))
def test_bin_settings_give_the_default_results(env, short_pairs, defaults):
    e = engine_with(env)
    try:
        assert flat(e.align_pairs(short_pairs, 1)) == defaults["binned"]
    finally:
        e.close()
