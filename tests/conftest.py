"""Shared fixtures of the GB300 NUFFT test-suite.

``-m "not gpu"`` runs the oracle against the golden vectors, the host-side
logic and the C-ABI load check; ``-m gpu`` runs the CUDA parity tests.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

GOLDEN = ROOT / "tests" / "golden" / "ndft_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libgbnufft.so")


@pytest.fixture(scope="session")
def pkg():
    return __graft_entry__.import_package()


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def gpu_pkg(pkg):
    """The package with its CUDA library built and loaded (GPU tests)."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    build = __graft_entry__._load_build_module()
    build.build()
    pkg.load_library()
    return pkg


def rel_l2(a, b):
    """Relative l2 error of ``a`` against reference ``b`` (same element count)."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.size == b.size, (a.shape, b.shape)
    a = a.reshape(b.shape)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
