"""Decoders on a cycle-free Tanner graph, against brute-force posteriors.

On a tree, layered belief propagation converges to the exact bitwise
posteriors: sum-product to the MAP LLRs, min-sum with scale 1 to the max-log
MAP LLRs.  This is the reference's own property test
(``tests/coding/test_ldpc.py:219-252``), here on a tree of our own: an
independent check of both the oracle (CPU) and the CUDA kernels (GPU) that
leans on neither of them.
"""

from __future__ import annotations

from itertools import product

import numpy as np
import pytest

import oracle

# Four checks on nine variables; the checks meet in variables 3, 1 and 5 only,
# so the check graph is the tree c1 - c0 - c2 plus c1 - c3.
ROWS = [[0, 1, 3], [3, 4, 5], [1, 2, 6], [5, 7, 8]]
N = 9


def _h():
    h = np.zeros((len(ROWS), N), np.int8)
    for i, r in enumerate(ROWS):
        h[i, r] = 1
    return h


def _brute_force(llrs):
    """Exact and max-log posteriors by enumerating every codeword; the
    channel LLR convention is ``log P(y|0) - log P(y|1)``."""
    h = _h()
    words = np.array([c for c in product((0, 1), repeat=N) if not (h @ np.array(c) % 2).any()])
    metric = -(llrs.astype(np.float64) @ words.T)  # log P(y | c) up to a constant
    exact = np.empty(llrs.shape, np.float64)
    maxlog = np.empty_like(exact)
    for i in range(N):
        zero, one = metric[:, words[:, i] == 0], metric[:, words[:, i] == 1]
        exact[:, i] = np.logaddexp.reduce(zero, axis=1) - np.logaddexp.reduce(one, axis=1)
        maxlog[:, i] = zero.max(axis=1) - one.max(axis=1)
    return exact, maxlog


def _llrs(frames=6, seed=11):
    return (1.2 * np.random.default_rng(seed).standard_normal((frames, N))).astype(np.float32)


def _tables():
    h = _h()
    row_ptr = np.concatenate([[0], np.cumsum(h.sum(1))]).astype(np.int32)
    cols = np.concatenate([np.nonzero(r)[0] for r in h]).astype(np.int32)
    return row_ptr, cols


def test_oracle_on_a_tree_is_exact():
    llrs = _llrs()
    exact, maxlog = _brute_force(llrs)
    row_ptr, cols = _tables()
    sp = oracle.decode(llrs, (row_ptr, cols, N), k=N - len(ROWS), sum_product=True,
                       max_iterations=10, early_stop=False)[1]  # fmt: skip
    ms = oracle.decode(llrs, (row_ptr, cols, N), k=N - len(ROWS), scale=1.0,
                       max_iterations=10, early_stop=False)[1]  # fmt: skip
    np.testing.assert_allclose(sp, exact, atol=2e-5)
    np.testing.assert_allclose(ms, maxlog, atol=2e-5)


@pytest.mark.gpu
def test_kernels_on_a_tree_are_exact():
    import torch

    import commkit_gb300 as ck

    llrs = _llrs()
    exact, maxlog = _brute_force(llrs)
    code = ck.LDPCCode.from_parity_check(_h())
    x = torch.from_numpy(llrs).cuda()
    sp = ck.decode(x, code=code, method=ck.SumProduct(max_iterations=10, early_stop=False))
    ms = ck.decode(x, code=code, method=ck.MinSum(scale=1.0, max_iterations=10, early_stop=False))
    np.testing.assert_allclose(sp.llrs.cpu().numpy(), exact, atol=2e-5)
    np.testing.assert_allclose(ms.llrs.cpu().numpy(), maxlog, atol=2e-5)
    # Bit-exact against the oracle as well, for min-sum.
    row_ptr, cols, _ = code._schedule
    want = oracle.decode(llrs, (row_ptr, cols, code.num_variables), k=code.k, scale=1.0,
                         max_iterations=10, early_stop=False)  # fmt: skip
    np.testing.assert_array_equal(ms.llrs.cpu().numpy(), want[1])
