"""Error of the decoder's posteriors against an FP64 evaluation of the same
layered min-sum.

``bench.decode_fp64`` evaluates the decode (schedule order, min1/min2/first
argmin, scale and offset, syndrome early stop) in float64 from the
decoder's float32 input LLRs.  Run in float32 it must equal the oracle bit
for bit, which pins its steps to the reference's; in float64 it is the
reference point for the error statement in the bench's parity blocks.  On
the GPU, the CUDA decoder is held to the oracle bit for bit elsewhere, so
its error against float64 is the oracle's, checked here."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from bench import decode_error_vs_fp64, decode_fp64
from commkit_gb300 import workloads as W
from commkit_gb300.coding import LDPCCode


def _case(name: str, frames: int, ebn0: float, seed: int):
    spec = W.CODES[name]
    code = LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    order = W.MIXED_ORDERS[name]
    b = W.coded_batch(spec, frames, order, ebn0, seed=seed)
    llr = np.stack([oracle.llr(b.symbols[f], order, oracle.inv_s2(b.noise_var[f])).reshape(-1)
                    for f in range(frames)])  # fmt: skip
    return code, llr


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build()


@pytest.mark.parametrize("name,ebn0,max_it", [("A", 1.2, 20), ("B", 5.4, 50)])
def test_float32_steps_equal_the_oracle(name, ebn0, max_it):
    code, llr = _case(name, 24, ebn0, seed=5)
    row, col, _ = code._schedule
    ob, opost, ov, oi = oracle.decode(llr, (row, col, code.num_variables), k=code.k, max_iterations=max_it)
    p32, i32, v32 = decode_fp64(llr, code._schedule, code.num_variables, 0.875, 0.0, max_it, dtype=np.float32)
    assert np.array_equal(p32, opost)
    assert np.array_equal(i32, oi)
    assert np.array_equal(v32, ov.astype(bool))
    assert not np.all(oi == max_it) and not np.all(oi < max_it)  # both outcomes occur


def test_converged_frames_agree_with_fp64():
    """Frames the float32 decode converges on take the same iteration count,
    validity and hard decisions in float64, with posteriors within a small
    fraction of the frame's largest |posterior|; the frames it cannot
    decode are only counted."""
    code, llr = _case("A", 48, 1.4, seed=9)
    row, col, _ = code._schedule
    ob, opost, ov, oi = oracle.decode(llr, (row, col, code.num_variables), k=code.k, max_iterations=20)
    e = decode_error_vs_fp64(opost, oi, ov, ob, code.k, llr, code._schedule, code.num_variables, 0.875, 0.0, 20)
    conv = e["converged"]
    print(e)
    assert conv["frames"] >= 24
    assert conv["same_iterations_and_valid"] == conv["frames"]
    assert conv["same_bits"] == conv["frames"]
    assert conv["max_rel_to_frame_peak"] < 0.02
    assert e["unconverged"]["frames"] + conv["frames"] == 48
