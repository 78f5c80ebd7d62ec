import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# compiled pass kernels are not cached on disk during the tests (the cache test sets
# its own directory); every test compiles what it runs
os.environ["QIBOJIT_GB300_CACHE"] = "0"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built engine library")


def pytest_generate_tests(metafunc):
    # the reference parametrises every state test over both complex precisions
    # (tests/conftest.py:35-39)
    if "dtype" in metafunc.fixturenames:
        metafunc.parametrize("dtype", ["complex128", "complex64"])


# Tolerances of the reference suite (tests/test_gates.py:15) for gate-level checks
# against dense matrices, and the engine's own kernel-parity bar: complex128 within
# 1e-12 max-abs of the oracle, complex64 within 1e-5.
ATOL = {"complex128": 1e-10, "complex64": 1e-4}
PARITY_ATOL = {"complex128": 1e-12, "complex64": 1e-5, "float64": 1e-12, "float32": 1e-5}
