"""Shared test set-up: import paths and the ``gpu`` marker.

Tests marked ``gpu`` need a CUDA device (a GB300) and the built libgnlm.so;
everything else runs on CPU.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "3d-gnlm_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def gnlm_lib():
    import gnlm
    if not os.path.exists(gnlm.LIB_PATH):
        gnlm.build()
    return gnlm
