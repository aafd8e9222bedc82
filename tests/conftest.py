"""Test configuration: the ``gpu`` marker and import paths.

``-m "not gpu"`` runs on any machine (oracle vs golden vectors, host planning, the C ABI's
exports). ``-m gpu`` needs a CUDA device and the built library; those tests call the stitching
kernels through the C ABI and check them against the oracle.
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
for p in (REPO, REPO / "hm-cupano_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libhmpano.so")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(REPO / "tests" / "golden" / "golden.npz")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle

    oracle.build()
    return oracle
