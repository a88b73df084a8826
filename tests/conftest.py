import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libogs_gpu.so")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (C restatement), built on first use."""
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu():
    """libogs_gpu.so loaded on a machine with a GPU (fails loudly otherwise)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected on a machine without CUDA")
    from ogs5_gb300 import build, capi
    build.build()
    capi.lib()
    return capi
