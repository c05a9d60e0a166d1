"""Host logic of the device encoder and the error-rate curve (CPU only):
which parity rule each code takes, the GF(2) inverse, and ErrorRateCurve's
validation and rates."""

from __future__ import annotations

import numpy as np
import pytest

from commkit_gb300 import ErrorRateCurve, LDPCCode
from commkit_gb300 import workloads as W
from commkit_gb300.coding import _gf2_inverse_packed
from tests.conftest import GOLDEN


def test_encoder_rules():
    for name in "ABC":
        code = LDPCCode.quasi_cyclic(W.CODES[name].base(), lifting=W.CODES[name].z)
        e = code._encoder
        assert e.stride == W.CODES[name].z and e.inverse is None
        assert e.info_row_ptr[-1] == np.count_nonzero(code.variables < code.k)
    d = np.load(GOLDEN / "dvbs2_normal.npz")
    code = LDPCCode(d["dvbs2n_checks"], d["dvbs2n_variables"], int(d["dvbs2n_m"]), int(d["dvbs2n_N"]))
    assert code._encoder.stride == 1
    g = np.load(GOLDEN / "ldpc_golden.npz")
    pon = LDPCCode(g["pon_checks"], g["pon_variables"], int(g["pon_m"]), int(g["pon_N"]),
                   int(g["pon_N"]) - int(g["pon_n"]))  # fmt: skip
    e = pon._encoder
    assert e.stride == 0 and e.inverse.shape == (pon.num_checks, (pon.num_checks + 31) // 32)


@pytest.mark.parametrize("m", [1, 31, 64, 100, 257])
def test_gf2_inverse(m):
    rng = np.random.default_rng(m)
    L = np.tril((rng.random((m, m)) < 0.1).astype(np.int64), -1) + np.eye(m, dtype=np.int64)
    U = np.triu((rng.random((m, m)) < 0.1).astype(np.int64), 1) + np.eye(m, dtype=np.int64)
    hp = (L @ U) % 2
    pr, pc = np.nonzero(hp)
    inv = _gf2_inverse_packed(pr, pc, m)
    bits = ((inv[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).reshape(m, -1)[:, :m].astype(np.int64)
    np.testing.assert_array_equal((hp @ bits) % 2, np.eye(m, dtype=np.int64))
    if m > 1:
        sing = hp.copy()
        sing[1] = sing[0]  # two equal rows
        with pytest.raises(NotImplementedError, match="singular"):
            _gf2_inverse_packed(*np.nonzero(sing), m)


def test_error_rate_curve_value():
    c = ErrorRateCurve([0.0, 1.0], num_blocks=[100, 200], bit_errors=[50, 10], block_errors=[20, 4],
                       pre_fec_bit_errors=[900, 700], detected_failures=[20, 4], undetected_errors=[0, 0],
                       total_iterations=[1000, 800], k=648, n=1296, bits_per_symbol=2)  # fmt: skip
    np.testing.assert_allclose(c.fer, [0.2, 0.02])
    np.testing.assert_allclose(c.ber, [50 / 64800, 10 / 129600])
    np.testing.assert_allclose(c.pre_fec_ber, [900 / 129600, 700 / 259200])
    np.testing.assert_allclose(c.mean_iterations, [10.0, 4.0])
    np.testing.assert_allclose(c.ebn0_db, c.esn0_db)  # rate 1/2, 2 bits per symbol
    with pytest.raises(ValueError, match="num_blocks"):
        ErrorRateCurve([0.0], num_blocks=[0], bit_errors=[0], block_errors=[0], pre_fec_bit_errors=[0],
                       detected_failures=[0], undetected_errors=[0], total_iterations=[0], k=1, n=2,
                       bits_per_symbol=1)  # fmt: skip
    with pytest.raises(ValueError, match="shape"):
        ErrorRateCurve([0.0, 1.0], num_blocks=[1], bit_errors=[0], block_errors=[0], pre_fec_bit_errors=[0],
                       detected_failures=[0], undetected_errors=[0], total_iterations=[0], k=1, n=2,
                       bits_per_symbol=1)  # fmt: skip
