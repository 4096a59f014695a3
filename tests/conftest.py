import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a) and the built libmeshode.so")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshode_gb300 import build as b
    b.build()
    return torch.device("cuda", 0)


@pytest.fixture(scope="session")
def orc():
    from oracle import pydeform_oracle
    pydeform_oracle.lib()
    return pydeform_oracle
