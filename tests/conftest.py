import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle and the CUDA library once per session (no-op when fresh)."""
    from conformal_cubed_sphere_gb300 import build as B
    from oracle import oracle as O
    O.build()
    B.build()
    yield
