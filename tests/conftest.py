"""Shared test set-up.

Markers: ``gpu`` tests need a CUDA device (sm_103a) and the built library;
everything else runs on the CPU.  The package directory
``fft-ocean-waves_gb300`` is not an importable name, so its modules are put
on sys.path directly.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fft-ocean-waves_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ocean_lib():
    """The built C-ABI library (built on demand; a build failure fails the test)."""
    import build as ocean_build
    ocean_build.build()
    import ocean_gb300
    ocean_gb300.load()
    return ocean_gb300


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
