"""Test configuration: paths, the ``gpu`` marker and shared helpers.

``-m gpu`` tests run the CUDA library on a GPU and compare it with the CPU
oracle (``oracle/``); the other tests check the oracle against the reference's
known answers and golden fixtures, and the host-side logic, without a GPU.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_PARENT = ROOT / "galaxy-collision-with-cuda-fft_gb300"
for p in (str(ROOT), str(PKG_PARENT)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libgcpm.so")
    config.addinivalue_line("markers", "slow: takes more than ~20 s on CPU")


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from galaxy_collision_gb300 import _build

    _build.build()
    return torch.device("cuda", 0)


def golden(name: str):
    return np.load(GOLDEN / name)


def gaussian_rho(n, dx, sigma, total_mass, center=None):
    """Normalised Gaussian density (mass/dx^3), the reference tests' fixture
    (tests/test_solver_multigrid.py:31-40)."""
    if center is None:
        axis = (np.arange(n) - (n - 1) / 2.0) * dx
        xx, yy, zz = np.meshgrid(axis, axis, axis, indexing="ij")
        r2 = xx**2 + yy**2 + zz**2
    else:
        axis = np.arange(n) * dx
        xx, yy, zz = np.meshgrid(axis, axis, axis, indexing="ij")
        r2 = (xx - center[0]) ** 2 + (yy - center[1]) ** 2 + (zz - center[2]) ** 2
    g = np.exp(-r2 / (2.0 * sigma**2))
    return (g / g.sum() * total_mass / dx**3).astype(np.float32)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
