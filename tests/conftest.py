"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs
on a CPU-only host."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build
    build()
    return Oracle()


@pytest.fixture(scope="session")
def gpu_icm():
    """The product package with its CUDA library built and a GPU selected."""
    from icm_gb300 import build as b
    b.build()
    import icm_gb300
    icm_gb300.init()
    return icm_gb300


def max_rel(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0
