import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # torch missing or broken: ask the driver through the engine instead
        return os.path.exists("/dev/nvidia0")


@pytest.fixture(scope="session")
def oracle_built():
    from oracle_lib import build_oracle

    build_oracle(with_ref=True)
    return True


@pytest.fixture(scope="session")
def engine():
    """The compiled engine library (built on first use). GPU tests fail loudly if it cannot be built."""
    from lmweather_gb300 import build

    build.build()
    import lmweather_gb300

    lmweather_gb300.load_library()
    return lmweather_gb300


def golden(name: str):
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", name))
