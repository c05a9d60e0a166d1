"""Codes whose parity part (the last m columns of H) is not invertible.

The reference encodes them through a systematic generator from H's reduced
row echelon form (its "dense" encoder, ``commkit/coding/ldpc.py:476-481``):
``k = N - rank(H)``, the information bits sit at the non-pivot columns, and
``decode`` takes its hard decisions there (``ldpc.py:582-586``).  The
fixtures (``ldpc_generator.npz``) hold the reference's own results on three
such codes.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300 import LDPCCode
from commkit_gb300.coding import _generator

NAMES = ("tree", "redundant", "qc_even")


@pytest.fixture(scope="module")
def golden():
    from tests.conftest import GOLDEN

    return np.load(GOLDEN / "ldpc_generator.npz")


def _code(g, name):
    return LDPCCode(g[f"{name}_checks"], g[f"{name}_variables"], int(g[f"{name}_m"]), int(g[f"{name}_N"]))


def _host_encode(code, u):
    """The device encoder's arithmetic on the host: information bits at the
    information columns, parity bit i = parity(generator row i AND u)."""
    info, piv, gen = _generator(code)
    k = code.k
    padded = np.zeros((u.shape[0], gen.shape[1] * 32), np.uint8)
    padded[:, :k] = u
    packed = np.packbits(padded, axis=1, bitorder="little").view(np.uint32)
    words = np.zeros((u.shape[0], code.num_variables), np.int8)
    words[:, info] = u
    both = gen[None, :, :] & packed[:, None, :]  # (frames, rank, words)
    ones = np.unpackbits(both.view(np.uint8), axis=2).sum(axis=2)
    words[:, piv] = (ones & 1).astype(np.int8)
    return words[:, : code.n]


@pytest.mark.parametrize("name", NAMES)
def test_generator_tables_match_reference(golden, name):
    code = _code(golden, name)
    assert code.k == int(golden[f"{name}_k"])
    np.testing.assert_array_equal(code._info, golden[f"{name}_info"])
    info, piv, gen = _generator(code)
    np.testing.assert_array_equal(piv, golden[f"{name}_pivots"])
    assert code._encoder.generator is not None
    words = _host_encode(code, golden[f"{name}_u"])
    np.testing.assert_array_equal(words, golden[f"{name}_words"])
    # Every word satisfies every check.
    syn = np.zeros((words.shape[0], code.num_checks), np.int64)
    np.add.at(syn.T, code.checks, words[:, code.variables].T.astype(np.int64))
    assert not np.any(syn % 2)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_decodes_match_reference(golden, name):
    code = _code(golden, name)
    row_ptr, cols, _ = code._schedule
    llrs = golden[f"{name}_llrs"]
    _, post, valid, iters = oracle.decode(llrs, (row_ptr, cols, code.num_variables), k=code.k)
    np.testing.assert_array_equal(post, golden[f"{name}_post"])
    np.testing.assert_array_equal(valid.astype(bool), golden[f"{name}_valid"])
    np.testing.assert_array_equal(iters, golden[f"{name}_iters"])
    np.testing.assert_array_equal((post[:, code._info] < 0).astype(np.int8), golden[f"{name}_bits"])


def test_leading_information_columns(golden):
    assert not _code(golden, "tree")._leading_info
    assert not _code(golden, "redundant")._leading_info
    # The circulant code's first k columns are independent of the rest.
    assert _code(golden, "qc_even")._leading_info


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_device_encode_and_decode_match_reference(golden, name):
    import torch

    import commkit_gb300 as ck

    code = _code(golden, name)
    dev = torch.device("cuda", 0)
    u = torch.from_numpy(golden[f"{name}_u"]).to(dev)
    words = ck.encode(u, code=code)
    np.testing.assert_array_equal(words.cpu().numpy(), golden[f"{name}_words"])
    llrs = torch.from_numpy(golden[f"{name}_llrs"]).to(dev)
    res = ck.decode(llrs, code=code, method=ck.MinSum())
    np.testing.assert_array_equal(res.llrs.cpu().numpy(), golden[f"{name}_post"])
    np.testing.assert_array_equal(res.bits.cpu().numpy(), golden[f"{name}_bits"])
    # One codeword per row: valid and iterations are (4, 1).
    np.testing.assert_array_equal(res.valid.cpu().numpy().reshape(-1), golden[f"{name}_valid"])
    np.testing.assert_array_equal(res.iterations.cpu().numpy().reshape(-1), golden[f"{name}_iters"])
    # Clean LLRs of a codeword decode back to its information bits.
    clean = 4.0 - 8.0 * words.float()
    back = ck.decode(clean, code=code)
    np.testing.assert_array_equal(back.bits.cpu().numpy(), golden[f"{name}_u"])
    assert bool(back.valid.all())


@pytest.mark.gpu
def test_mixed_forms_refuse_scattered_information_columns(golden):
    import torch

    import commkit_gb300 as ck

    code = _code(golden, "tree")
    x = torch.zeros((2, code.n), device="cuda")
    with pytest.raises(NotImplementedError, match="not the first k"):
        ck.decode_mixed([(x, code, ck.MinSum())])
    # A circulant code whose first k columns are the information takes the mixed path.
    qc = _code(golden, "qc_even")
    llrs = torch.from_numpy(golden["qc_even_llrs"]).cuda()
    (mixed,) = ck.decode_mixed([(llrs, qc, ck.MinSum())])
    plain = ck.decode(llrs, code=qc)
    for a, b in ((mixed.bits, plain.bits), (mixed.llrs, plain.llrs), (mixed.iterations, plain.iterations)):
        assert torch.equal(a.reshape(-1), b.reshape(-1))
