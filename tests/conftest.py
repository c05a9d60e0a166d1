"""Test configuration: the ``gpu`` marker and shared fixtures.

``pytest -m "not gpu"`` runs on any machine: the oracle against the golden
fixtures, the host logic, and that the C-ABI library loads and exports its
symbols.  ``pytest -m gpu`` runs the parity tests of the CUDA path against
the oracle, through the C ABI; they need a CUDA device and the library
built (``python -c "import __graft_entry__ as g; g.build()"``).
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (sm_103a) and the built library")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def golden_qam():
    return dict(np.load(GOLDEN / "qam_tables.npz"))


@pytest.fixture(scope="session")
def golden_llr():
    return dict(np.load(GOLDEN / "llr_golden.npz"))


@pytest.fixture(scope="session")
def golden_ldpc():
    return dict(np.load(GOLDEN / "ldpc_golden.npz"))


def digest(a: np.ndarray) -> str:
    """SHA-256 of an array's bytes with negative zeros folded to +0, the
    digest ``tests/golden/make_golden.py`` stores."""
    import hashlib

    a = np.ascontiguousarray(a)
    if a.dtype.kind == "f":
        a = np.where(a == 0, np.zeros_like(a), a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def kat_llrs(n: int) -> np.ndarray:
    """The reference's KAT input: ``1.8 + 1.5 N(0,1)``, 6 frames, seed 1
    (``tests/coding/test_ldpc_kernel.py:16-18``)."""
    rng = np.random.default_rng(1)
    return (1.8 + 1.5 * rng.standard_normal((6, n))).astype(np.float32)
