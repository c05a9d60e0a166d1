"""The per-call extension (``csrc/python/ck_calls.cpp``) on the CPU: it loads
against this torch, and every call it must not take comes back as None, so
the public functions fall through to their general path and its errors."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import commkit_gb300 as ck
from commkit_gb300 import _lib, coding, mapping
from commkit_gb300 import workloads as W


@pytest.fixture(scope="module")
def calls():
    mod = _lib.calls()
    assert mod is not None, f"{_lib.CALLS_PATH} was not built or does not load"
    return mod


def test_loads_and_exports(calls):
    for name in ("init", "decode", "llr", "release", "workspaces"):
        assert callable(getattr(calls, name))
    assert calls.workspaces() == []  # nothing decoded on this CPU-only host


def test_declines_what_it_does_not_take(calls):
    call = (0, 0.875, 0.0, 20, 1)
    entries = [(1 << 20, 8, 4)]  # never dereferenced: every call below is declined first
    for x in (torch.zeros(16), torch.zeros(16, dtype=torch.float64), np.zeros(16, np.float32), None, 3.0):
        assert calls.decode(x, entries, call) is None
    table = [(0, 0, 1 << 20, 1 << 21, 0, 0, 4)]
    for x in (torch.zeros(8, dtype=torch.complex64), torch.zeros(8), np.zeros(8, np.complex64)):
        assert calls.llr(x, 0.5, table) is None


def test_rejects_malformed_calls(calls):
    with pytest.raises(TypeError):
        calls.decode(torch.zeros(4), [], (0, 1.0, 0.0))
    with pytest.raises(TypeError):
        calls.decode(torch.zeros(4), (), (0, 1.0, 0.0, 1, 1))
    with pytest.raises(TypeError):
        calls.llr(torch.zeros(4, dtype=torch.complex64), 0.5)
    with pytest.raises(TypeError):
        calls.init(1, 2, 3)


def test_registered_forms_fall_through_to_the_general_path(calls):
    """With entries registered (as a GPU call would leave them), host input
    still reaches the general path and its errors."""
    # Fresh objects (the factories cache theirs), and the fake entries, whose
    # addresses hold no tables, are taken out again.
    q = ck.Constellation.qam(16)
    c = ck.Constellation(q.points, q.bit_labels)
    c.__dict__["_calls_llr"] = {"maxlog": [(0, 0, 1 << 20, 1 << 21, 0, 0, 4)]}
    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    code._calls_entries = [(1 << 20, code.n, code.k)]
    saved = coding._calls_decode
    try:
        with pytest.raises(TypeError, match="CUDA"):
            ck.compute_llr(torch.zeros(8, dtype=torch.complex64), noise_var=0.5, constellation=c)
        with pytest.raises(TypeError, match="CUDA"):
            c.llr(torch.zeros(8, dtype=torch.complex64), noise_var=0.5)
        assert mapping._calls_llr(torch.zeros(8, dtype=torch.complex64), 0.5, c, ["maxlog"]) is None
        assert mapping._calls_llr(torch.zeros(8, dtype=torch.complex64), 0.5, None, "maxlog") is None

        coding._rule_args(coding._DEFAULT_METHOD)
        coding._calls_decode = calls.decode
        with pytest.raises(TypeError, match="CUDA"):
            ck.decode(torch.zeros(code.n), code=code)
        with pytest.raises(TypeError, match="method"):
            ck.decode(torch.zeros(code.n), code=code, method="min-sum")
    finally:
        del c.__dict__["_calls_llr"]
        code._calls_entries = None
        coding._calls_decode = saved


def test_method_call_tuple():
    m = ck.MinSum(scale=0.75, offset=0.125, max_iterations=7, early_stop=False)
    assert coding._rule_args(m) == (_lib.CK_LDPC_MIN_SUM, 0.75, 0.125)
    assert m.__dict__["_c_call"] == (_lib.CK_LDPC_MIN_SUM, 0.75, 0.125, 7, 0)
    s = ck.SumProduct(max_iterations=9)
    coding._rule_args(s)
    assert s.__dict__["_c_call"] == (_lib.CK_LDPC_SUM_PRODUCT, 1.0, 0.0, 9, 1)
