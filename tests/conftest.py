import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs through the C ABI library")


@pytest.fixture(scope="session")
def oracle_lib():
    """The CPU restatement (oracle/_build/liboracle_flip.so), built on first use."""
    from oracle import bindings as B
    if not os.path.exists(B.ORACLE_SO):
        B.build(ref=False)
    return B


@pytest.fixture(scope="session")
def flip_lib():
    """The CUDA library, built in-tree on first use (cross-compiles without a GPU)."""
    from vare_gb300 import build, flip
    build.build()
    return flip


@pytest.fixture(scope="session")
def gpu(flip_lib):
    """Skip unless a CUDA device is present; the library must then be the one that runs."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return flip_lib
