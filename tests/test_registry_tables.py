"""This package's host side against the reference's recorded launcher calls
(``registry_calls.npz``, CPU): for each recorded demapper call, the kernel
this package routes the constellation and method to, its host tables and the
``inv_s2`` it derives from ``esn0_db`` (bit for bit, as float32) equal what
the reference passed; for each recorded decode, the first-fit schedule
equals the reference's."""

from __future__ import annotations

import numpy as np
import pytest

from commkit_gb300 import workloads as W
from commkit_gb300.mapping import Constellation, _noise_variance, _table_kind, host_tables, inv_s2
from tests.conftest import GOLDEN
from tests.golden.make_golden import REGISTRY_LDPC_CASES, REGISTRY_LLR_CASES

KERNEL_OF_KIND = {"maxlog": "llr_separable_maxlog", "levels": "llr_separable", "points": "llr"}


@pytest.fixture(scope="module")
def calls():
    return dict(np.load(GOLDEN / "registry_calls.npz"))


def _constellation(kind):
    family, order = kind
    if family == "qam":
        return Constellation.qam(order)
    if family == "psk":
        return Constellation.psk(order)
    return Constellation.qam(order).shaped(entropy=3.5)


@pytest.mark.parametrize("case", REGISTRY_LLR_CASES, ids=[c[0] for c in REGISTRY_LLR_CASES])
def test_demapper_routing_tables_and_inv_s2(calls, case):
    tag, kind, method, esn0, _ = case
    g = calls
    c = _constellation(kind)
    tk = _table_kind(c, method)
    assert KERNEL_OF_KIND[tk] == str(g[f"{tag}_name"])
    ours = host_tables(c, tk)
    if tk == "points":
        want = [g[f"{tag}_arg{j}"] for j in range(3)]
    else:
        want = [g[f"{tag}_arg{j}_{t}"] for j in range(2) for t in range(int(g[f"{tag}_arg{j}_len"]))]
    assert len(ours) == len(want)
    for a, b in zip(ours, want, strict=True):
        assert a.dtype == b.dtype
        np.testing.assert_array_equal(a, b)
    s2 = inv_s2(_noise_variance(None, esn0, c, False, "compute_llr()"))
    assert np.float32(s2).tobytes() == np.float32(g[f"{tag}_kw_inv_s2"]).tobytes()
    if tk == "points":
        assert int(g[f"{tag}_kw_k"]) == c.bits_per_symbol


@pytest.mark.parametrize("case", REGISTRY_LDPC_CASES, ids=[c[0] for c in REGISTRY_LDPC_CASES])
def test_decoder_schedule(calls, golden_ldpc, case):
    import commkit_gb300 as ck

    tag, which = case[0], case[1]
    g = calls
    if which == "A":
        code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    else:
        m, N, n = (int(golden_ldpc[f"{which}_{s}"]) for s in ("m", "N", "n"))
        code = ck.LDPCCode(golden_ldpc[f"{which}_checks"], golden_ldpc[f"{which}_variables"], m, N, N - n)
    row_ptr, cols, layer_ptr = code._schedule
    np.testing.assert_array_equal(row_ptr, g[f"{tag}_row_ptr"])
    np.testing.assert_array_equal(cols, g[f"{tag}_cols"])
    np.testing.assert_array_equal(layer_ptr, g[f"{tag}_layer_ptr"])
    assert code.n == int(g[f"{tag}_n"]) and code.num_variables == int(g[f"{tag}_N"])
