import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: full-size case (seconds to a minute)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the product library and the CPU oracle once per session (CPU-only steps)."""
    from pmdas_gb300 import build as B
    from oracle import build as OB
    B.build()
    OB.build_oracle()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
