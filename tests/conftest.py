import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
ORACLE = os.path.join(REPO, "oracle")
if ORACLE not in sys.path:
    sys.path.insert(0, ORACLE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def orc():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def tc():
    """The CUDA library, built in-tree if needed (GPU tests only)."""
    from fft_demo_gb300 import build as b
    b.build()
    import fft_demo_gb300
    fft_demo_gb300.lib()
    return fft_demo_gb300


def uniform_complex(rng, shape, lo=-1.0, hi=1.0):
    return rng.uniform(lo, hi, shape) + 1j * rng.uniform(lo, hi, shape)
