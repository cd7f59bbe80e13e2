import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """Builds libpct_gb300.so and the oracle once per session (no-op when up to date)."""
    from pct_gb300 import build as pbuild
    from oracle import build_oracle
    pbuild.build()
    build_oracle.build()
    yield


def has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
