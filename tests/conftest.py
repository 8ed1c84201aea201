"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built libc3d.so;
everything else runs on CPU (oracle known-answer tests, C-ABI symbol checks, host logic)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libc3d.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def rel_l2(a, b):
    import numpy as np
    den = float(np.sqrt(np.sum(b * b)))
    return float(np.sqrt(np.sum((a - b) ** 2))) / max(den, 1e-300)
