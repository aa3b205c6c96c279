import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")
GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")
if GOLDEN_DIR not in sys.path:
    sys.path.insert(0, GOLDEN_DIR)
DIGESTS = os.path.join(GOLDEN_DIR, "workload_digests.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O.Oracle()


@pytest.fixture(scope="session")
def reference():
    """The unmodified reference (only where its checkout exists and built); otherwise the test is skipped."""
    from oracle import oracle as O
    try:
        O.build()
        return O.Reference()
    except (FileNotFoundError, OSError, Exception) as e:  # noqa: BLE001
        pytest.skip(f"reference build unavailable: {e}")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def ref_digests():
    """Digests of the reference's outputs on the benchmark workloads (tests/golden/make_workload_digests.py)."""
    return np.load(DIGESTS)


def ragged(z, name, i):
    off = z[name + "_off"]
    return z[name][off[i]:off[i + 1]]


@pytest.fixture(scope="session")
def lib():
    """The product library (CUDA path).  GPU tests only."""
    import dcns_gb300
    dcns_gb300.build()
    return dcns_gb300.load()
