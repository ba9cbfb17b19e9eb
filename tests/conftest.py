"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built liblexgb.so")


def report_path(name):
    """Where the GPU tests write their JSON reports: $LEXGB_REPORT_DIR, else reports/ in the repo."""
    d = os.environ.get("LEXGB_REPORT_DIR") or os.path.join(ROOT, "reports")
    os.makedirs(d, exist_ok=True)
    return os.path.join(d, name)


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def ops_golden():
    return load_golden("ops_random.npz")


@pytest.fixture(scope="session")
def bubble_golden():
    return load_golden("bubble_steps.npz")


@pytest.fixture(scope="session")
def built_lib():
    """Build (incrementally) and load the native library; GPU tests only."""
    from lex_gb300 import build, _lib
    build.build()
    return _lib.load()


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
