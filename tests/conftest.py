import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(__file__))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (runs through the C ABI of libkm_sm103)")


@pytest.fixture(scope="session")
def km():
    import helpers
    return helpers.km()


@pytest.fixture(scope="session")
def gpu(km):
    import torch
    if not torch.cuda.is_available() or km.device_count() == 0:
        pytest.fail("GPU test run without an sm_103 device")
    torch.cuda.init()
    return torch.device("cuda:0")
