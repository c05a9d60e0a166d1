"""Host-side logic and the C-ABI library, without a GPU."""

from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from commkit_gb300 import LDPCCode, MinSum, SumProduct, _lib, workloads as W
from commkit_gb300.mapping import Constellation, _noise_variance, inv_s2

ROOT = Path(__file__).resolve().parents[1]


def _declared_functions() -> list[str]:
    text = (ROOT / "include" / "commkit_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ck_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    declared = _declared_functions()
    assert declared, "no declarations found"
    assert sorted(_lib.EXPORTS) == declared
    for name in declared:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout  # fmt: skip
    exported = set(re.findall(r"\bT (ck_[a-z0-9_]+)", out))
    assert set(declared) <= exported
    assert lib.ck_version() == b"0.1.0"
    assert lib.ck_status_string(5) == b"device-side wait timed out"


def test_python_constants_equal_the_header():
    """Every integer #define of the C header has the same value in _lib."""
    text = (ROOT / "include" / "commkit_gb300.h").read_text()
    found = re.findall(r"#define (CK_[A-Z0-9_]+) \(?([0-9u* ]+)\)?", text)
    assert len(found) > 10
    for name, value in found:
        want = 1
        for factor in value.replace("u", "").split("*"):
            want *= int(factor)
        assert getattr(_lib, name) == want, name


def test_feed_frame_layout_and_host_publish():
    """The continuous feed's descriptor as the C header declares it (five
    pointers, a float, a word: 48 bytes), and the host side of a feed, which
    needs no GPU: ck_ldpc_feed_publish writes a request's descriptors around
    the end of the ring, sets its iteration slots to -2 and raises the
    published count."""
    F = _lib.FeedFrame
    assert ctypes.sizeof(F) == 48
    assert [getattr(F, n).offset for n, _ in F._fields_] == [0, 8, 16, 24, 32, 40, 44]
    assert ctypes.sizeof(_lib.FeedRing) == 24
    cap, n_in, k_bits = 8, 100, 40
    ring = (F * cap)()
    iters = (ctypes.c_int32 * cap)(*range(cap))
    published = ctypes.c_uint32(6)
    sym, llr, bits, valid = 1 << 20, 2 << 20, 3 << 20, 4 << 20
    st = _lib.lib().ck_ldpc_feed_publish(ctypes.addressof(ring), cap, ctypes.addressof(iters),
                                         ctypes.addressof(published), 6, 4, sym, 4096, llr, n_in, bits, k_bits,
                                         valid, 0.25, 77)  # fmt: skip
    assert st == 0
    assert published.value == 10
    for f, slot in enumerate([6, 7, 0, 1]):
        d = ring[slot]
        assert d.symbols == sym + 4096 * f and d.llr_out == llr + 4 * n_in * f
        assert d.bits == bits + k_bits * f and d.valid == valid + f
        assert d.iters == ctypes.addressof(iters) + 4 * slot and iters[slot] == -2
        assert d.inv_s2 == 0.25 and d.seq == 77 + f
    assert [iters[s] for s in (2, 3, 4, 5)] == [2, 3, 4, 5]
    assert _lib.lib().ck_ldpc_feed_publish(ctypes.addressof(ring), 6, ctypes.addressof(iters),
                                           ctypes.addressof(published), 0, 1, sym, 8, llr, n_in, None, 0, valid,
                                           1.0, 0) != 0  # capacity not a power of two  # fmt: skip
    word = (ctypes.c_uint32 * 2)(7, 9)
    _lib.lib().ck_host_publish(ctypes.addressof(word), 12345)
    assert list(word) == [12345, 9]


@pytest.mark.parametrize("name", ["A", "B", "C"])
def test_native_schedule_matches_oracle(name):
    spec = W.CODES[name]
    base = spec.base()
    code = LDPCCode.quasi_cyclic(base, lifting=spec.z)
    got = code._schedule
    want = oracle.schedule(code.checks, code.variables, code.num_checks, code.num_variables)
    for a, b in zip(got, want, strict=True):
        np.testing.assert_array_equal(a, b)


def test_native_schedule_matches_oracle_kats(golden_ldpc):
    for which in ("dvbs2s", "pon"):
        m, N = int(golden_ldpc[f"{which}_m"]), int(golden_ldpc[f"{which}_N"])
        code = LDPCCode(golden_ldpc[f"{which}_checks"], golden_ldpc[f"{which}_variables"], m, N,
                        N - int(golden_ldpc[f"{which}_n"]))  # fmt: skip
        want = oracle.schedule(code.checks, code.variables, m, N)
        for a, b in zip(code._schedule, want, strict=True):
            np.testing.assert_array_equal(a, b)
        assert code.k == int(golden_ldpc[f"{which}_k"])


def test_schedule_rejects_bad_edges():
    lib = _lib.lib()
    checks = np.array([0, 0, 1, 1], np.int32)
    variables = np.array([1, 0, 0, 1], np.int32)  # row 0 not sorted
    buf = [np.zeros(3, np.int32), np.zeros(4, np.int32), np.zeros(3, np.int32)]
    num = ctypes.c_int32()
    st = lib.ck_ldpc_schedule(checks.ctypes.data, variables.ctypes.data, 4, 2, 3,
                              *[b.ctypes.data for b in buf], ctypes.byref(num))  # fmt: skip
    assert st == _lib.CK_ERR_INVALID_ARGUMENT
    assert "sorted" in _lib.last_error()


def test_codes_have_the_configured_shapes():
    a, b, c = (LDPCCode.quasi_cyclic(s.base(), lifting=s.z) for s in (W.CODE_A, W.CODE_B, W.CODE_C))
    assert (a.num_variables, a.k, a.n) == (1296, 648, 1296)
    assert (b.num_variables, b.k) == (2304, 1728)
    assert (c.num_variables, c.k, c.num_checks) == (26112, 8448, 17664)
    assert np.count_nonzero(W.CODE_C.base() >= 0) == round(0.1 * 46 * 68)
    cw = (W.CODE_A.base()[:, :12] >= 0).sum(axis=0)
    assert sorted(cw.tolist()) == [3] * 6 + [6] * 6


@pytest.mark.parametrize("spec", [W.CODE_A, W.CODE_B, W.CODE_C], ids=["A", "B", "C"])
def test_workload_codewords_satisfy_every_check(spec):
    base = spec.base()
    info = np.random.default_rng(1).integers(0, 2, (3, (base.shape[1] - base.shape[0]) * spec.z),
                                             dtype=np.int8)  # fmt: skip
    words = W.encode_qc(base, spec.z, info)
    checks, variables = W.lift(base, spec.z)
    m = base.shape[0] * spec.z
    syn = np.zeros((3, m), np.int64)
    np.add.at(syn.T, checks, words[:, variables].T.astype(np.int64))
    assert not (syn % 2).any()
    np.testing.assert_array_equal(words[:, : info.shape[1]], info)


def test_code_validation():
    with pytest.raises(ValueError, match="duplicate"):
        LDPCCode(np.array([0, 0, 0, 1, 1]), np.array([0, 0, 1, 1, 2]), 2, 4)
    with pytest.raises(ValueError, match="two bits"):
        LDPCCode(np.array([0, 0, 1]), np.array([0, 1, 2]), 2, 4)
    with pytest.raises(ValueError, match="out of range"):
        LDPCCode(np.array([0, 0]), np.array([0, 9]), 1, 4)
    with pytest.raises(ValueError, match="shifts"):
        LDPCCode.quasi_cyclic(np.array([[0, -2]]), lifting=3)
    with pytest.raises(ValueError):
        LDPCCode.quasi_cyclic(np.array([[0, 1]]), lifting=0)
    with pytest.raises(ValueError, match="parity bits"):
        LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=54, punctured=700)


def test_method_validation():
    with pytest.raises(ValueError):
        MinSum(scale=0.0)
    with pytest.raises(ValueError):
        MinSum(scale=1.5)
    with pytest.raises(ValueError):
        MinSum(offset=-1.0)
    with pytest.raises(ValueError):
        MinSum(max_iterations=0)
    with pytest.raises(ValueError):
        MinSum(max_iterations=True)
    with pytest.raises(ValueError):
        SumProduct(max_iterations=-3)


def test_noise_variance_rules():
    c = Constellation.qam(16)
    assert _noise_variance(0.1, None, c, False, "f") == 0.1
    assert _noise_variance(None, 10.0, c, False, "f") == pytest.approx(c.power() / 10.0)
    assert _noise_variance(None, 10.0, c, True, "f") == pytest.approx(c.power() / 20.0)
    with pytest.raises(ValueError, match="one of"):
        _noise_variance(None, None, c, False, "f")
    with pytest.raises(ValueError, match="one of"):
        _noise_variance(0.1, 3.0, c, False, "f")
    assert inv_s2(0.0) == float(np.float32(1e20))
    assert inv_s2(0.1) == float(np.float32(10.0))


def test_host_input_is_rejected():
    """No CPU path: host arrays raise TypeError before any device work."""
    import commkit_gb300 as ck

    code = LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=54)
    with pytest.raises(TypeError, match="CUDA"):
        ck.decode(np.zeros(code.n, np.float32), code=code)
    with pytest.raises(TypeError, match="CUDA"):
        ck.compute_llr(np.zeros(4, np.complex64), noise_var=0.1, constellation=Constellation.qam(16))


def test_fastdiv_exhaustive_on_host():
    """The multiply-high division the kernels use (ck_common.cuh), restated
    here and checked for the divisors and ranges the decoder meets."""
    def make(d):
        l = 0
        while (1 << l) < d:
            l += 1
        mul = ((1 << 32) * ((1 << l) - d)) // d + 1
        return mul & 0xFFFFFFFF, l

    rng = np.random.default_rng(0)
    for d in [1, 2, 3, 7, 54, 96, 256, 360, 384, 1000, 4097, 65535, 1 << 20]:
        mul, sh = make(d)
        n = np.concatenate([np.arange(0, 70000, dtype=np.uint64),
                            rng.integers(0, 2**31, 200000, dtype=np.uint64)])  # fmt: skip
        hi = (n * np.uint64(mul)) >> np.uint64(32)
        q = (hi + n) >> np.uint64(sh)
        np.testing.assert_array_equal(q, n // np.uint64(d))


def test_four_cycle_warning_and_sparse_parity_check(caplog):
    """``LDPCCode.from_parity_check`` takes dense or SciPy sparse 0/1
    matrices and, like ``quasi_cyclic``, logs a warning when two checks
    share two bits (``commkit/coding/ldpc.py:146-181, 415-419``)."""
    import logging

    import scipy.sparse

    from commkit_gb300.coding import LDPCCode

    cyc = np.array([[1, 1, 1, 0], [1, 1, 0, 1], [0, 0, 1, 1]])  # checks 0 and 1 share bits 0 and 1
    tree = np.array([[1, 1, 0, 0], [0, 1, 1, 0], [0, 0, 1, 1]])
    with caplog.at_level(logging.WARNING, logger="commkit_gb300.coding"):
        a = LDPCCode.from_parity_check(cyc)
        assert any("4-cycles" in r.getMessage() for r in caplog.records)
        caplog.clear()
        b = LDPCCode.from_parity_check(scipy.sparse.csr_array(tree))
        assert not any("4-cycles" in r.getMessage() for r in caplog.records)
    assert (a.num_checks, a.num_variables) == (3, 4)
    c = LDPCCode.from_parity_check(tree)
    assert np.array_equal(b._schedule[1], c._schedule[1]) and b.k == c.k
    with pytest.raises(ValueError, match="only 0 and 1"):
        LDPCCode.from_parity_check(scipy.sparse.csr_array(2 * tree))
