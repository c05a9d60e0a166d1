"""Error of the LLRs against an FP64 evaluation of the same formula.

The float64 evaluation (``bench.llr_fp64``) takes the kernel's float32 inputs
(symbols, points, log prior, inv_s2) and carries the metric, the maxima and
the log-sum-exp in double precision.  On the CPU it bounds the oracle's own
float32 error; on the GPU every LLR must be no further from it than the
reference's float32 evaluation is, plus the parity tolerance (1e-5 relative,
1e-6 absolute), and the test prints the largest errors it saw."""

from __future__ import annotations

import numpy as np
import pytest

from bench import llr_error_vs_fp64, llr_fp64
from commkit_gb300.mapping import Constellation, inv_s2
from tests.test_constellations import oracle_llr

CASES = {
    "qam16": lambda: Constellation.qam(16),
    "qam64": lambda: Constellation.qam(64),
    "psk16": lambda: Constellation.psk(16),
    "qam8": lambda: Constellation.qam(8),
    "qam128_cross": lambda: Constellation.qam(128),
    "qam64_shaped": lambda: Constellation.qam(64).shaped(entropy=5.0),
}


def symbols(c: Constellation, n: int, sigma: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = c.points[rng.integers(0, c.order, n)] + sigma * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    return x.astype(np.complex64)


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("method", ["maxlog", "exact"])
def test_oracle_against_fp64(name, method):
    """The float32 oracle (the reference's formula and order) stays within
    a few float32 rounding steps of the float64 evaluation."""
    c = CASES[name]()
    for nv, seed in ((0.05, 1), (0.5, 2)):
        x = symbols(c, 2048, np.sqrt(nv / 2), seed)
        got = oracle_llr(c, x, nv, method).reshape(x.size, -1)
        ref = llr_fp64(x, c, np.full(x.size, inv_s2(nv), np.float32), method == "exact")
        err = llr_error_vs_fp64(got, ref)
        assert err["max_abs"] < 1e-4 and err["max_rel"] < 1e-4, err


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("method", ["maxlog", "exact"])
def test_gpu_against_fp64(name, method):
    import torch

    import commkit_gb300 as ck

    c = CASES[name]()
    for nv, seed in ((0.05, 3), (0.5, 4)):
        x = symbols(c, 1 << 14, np.sqrt(nv / 2), seed)
        got = ck.compute_llr(torch.from_numpy(x).cuda(), noise_var=nv, constellation=c, method=method)
        got = got.cpu().numpy().reshape(x.size, -1).astype(np.float64)
        ref = llr_fp64(x, c, np.full(x.size, inv_s2(nv), np.float32), method == "exact")
        cpu = oracle_llr(c, x, nv, method).reshape(x.size, -1).astype(np.float64)
        bound = np.abs(cpu - ref) + 1e-5 * np.abs(ref) + 1e-6
        assert np.all(np.abs(got - ref) <= bound)
        print(f"{name} {method} nv={nv}: GPU vs fp64 {llr_error_vs_fp64(got, ref)}, "
              f"oracle vs fp64 {llr_error_vs_fp64(cpu, ref)}")
