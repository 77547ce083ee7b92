"""Shared fixtures. ``gpu`` marks tests that need a GB300 (run with ``-m gpu``)."""

from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103a)")


@pytest.fixture(scope="session")
def port():
    import oracle

    oracle.build(reference=False)
    return oracle.Oracle("port")


@pytest.fixture(scope="session")
def reference():
    """The reference's own core compiled from its sources (skipped where absent)."""

    import oracle

    if not oracle.reference_available():
        try:
            oracle.build(reference=None)
        except Exception:
            pass
    if not oracle.reference_available():
        pytest.skip("reference sources not present on this machine")
    return oracle.Oracle("reference")


@pytest.fixture(scope="session")
def backend():
    import mpsboost_gb300 as mb

    return mb.CudaBackend(0)


def seeded_matrix(seed: int, rows: int, features: int, nan_fraction: float = 0.0,
                  integer_columns: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(rows, features)).astype(np.float32)
    for c in range(min(integer_columns, features)):
        x[:, c] = rng.integers(0, 2 + 3 * c, rows).astype(np.float32)
    if nan_fraction:
        x[rng.random((rows, features)) < nan_fraction] = np.nan
    return x
