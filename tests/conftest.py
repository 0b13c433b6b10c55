"""Shared test set-up: import paths, the `gpu` marker, helpers.

CPU tests (-m "not gpu") check the oracle against the reference's golden
vectors and known answers, the host logic, and that the C-ABI library exports
every declared symbol.  GPU tests (-m gpu) run the CUDA library through its
C-ABI and compare with the oracle on the same seeded inputs.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "astraea-impact-sim_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def rel_rms(a, b):
    """Norm-relative RMS difference sqrt(sum (a-b)^2 / sum b^2)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b * b), 1e-300)))


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")
