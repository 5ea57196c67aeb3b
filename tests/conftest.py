import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libslg.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library; GPU tests fail (not skip) when it cannot be loaded."""
    import softlight_gb300 as sg
    sg.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return sg


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_oracle()
    return oracle
