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


@pytest.fixture(scope="session")
def golden_sp():
    return dict(np.load(GOLDEN / "ldpc_sp_golden.npz"))


# Sum-product cases of ldpc_sp_golden.npz, and which of them run on past the
# point where posteriors saturate.
SP_TAGS = ("dvbs2s", "pon", "dvbs2s_hi", "pon_hi")
SP_SATURATED = ("dvbs2s_hi",)


def check_sum_product(g: dict, key: str, bits, post, valid, iters, *, saturated: bool) -> None:
    """A sum-product decode against a fixture: hard decisions, syndrome flags
    and iteration counts exactly; posteriors at the reference's own GPU-vs-CPU
    tolerance, rtol = atol = 1e-3 (``tests/coding/test_ldpc_kernel.py:37-45``).

    Where frames converge (``saturated``), |LLR| grows past 10 and
    phi(x) = -log tanh(x/2) is evaluated where tanh(x/2) lies within a few
    ulps of 1: phi of a large argument is then quantised to multiples of
    ~6e-8, and phi of the difference of two such totals, ~-log(y/2) for a
    tiny y, moves by up to ln 2 = 0.69 when y doubles.  Any two float32
    evaluations of tanh and log (the reference's NumPy, C's libm, CUDA's)
    therefore differ there by up to ~0.7 per incoming message.  Such
    posteriors are held to the same sign, a median relative error of 1% and
    a largest relative error of 15% (seen: 5.6% between the reference and the
    C oracle, 9.3% between the GPU and the oracle on code C).
    """
    np.testing.assert_array_equal(np.asarray(iters).reshape(-1), g[key + "_iters"], err_msg="iterations")
    np.testing.assert_array_equal(np.asarray(valid).reshape(-1), g[key + "_valid"], err_msg="valid")
    packed = np.packbits(np.asarray(bits, np.uint8).reshape(g[key + "_post"].shape[0], -1), axis=1)
    np.testing.assert_array_equal(packed, g[key + "_bits_packed"], err_msg="bits")
    ref = g[key + "_post"]
    post = np.asarray(post, np.float32).reshape(ref.shape)
    if saturated:
        assert np.array_equal(np.signbit(post), np.signbit(ref))
        rel = np.abs(post - ref) / np.maximum(np.abs(ref), 1e-30)
        assert np.median(rel) <= 1e-2 and rel.max() <= 0.15, (np.median(rel), rel.max())
    else:
        np.testing.assert_allclose(post, ref, rtol=1e-3, atol=1e-3)


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
