"""Codes with rows above 27 edges on the GPU: the any-degree kernels (wide
min-sum state, generic row loop) against the reference's own decodes
(``ldpc_wide.npz``: DVB-S2 normal 9/10 with rows of 30 edges, and two
seeded codes with rows of 64, circulant and not).  Min-sum is bit-exact;
sum-product at the reference's tolerance (``check_sum_product``).  The
reference decodes any row degree (``commkit/_cuda/src/ldpc.cu:45-91``,
``commkit/coding/_numba_loops.py:43-94``)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.conftest import GOLDEN, check_sum_product, digest
from tests.golden.make_golden import wide_llrs

pytestmark = pytest.mark.gpu

NAMES = ("w64qc", "w64csr", "dvbs2n910")
TAGS = ("ms", "ms2", "sp0", "sp1")


@pytest.fixture(scope="module")
def golden_wide():
    return dict(np.load(GOLDEN / "ldpc_wide.npz"))


@pytest.fixture(scope="module")
def torch_dev():
    import torch

    return torch, torch.device("cuda", 0)


@pytest.fixture(scope="module")
def ck():
    import commkit_gb300

    return commkit_gb300


def _code(ck, g, name):
    m, N, n = (int(g[f"{name}_{s}"]) for s in ("m", "N", "n"))
    return ck.LDPCCode(g[f"{name}_checks"], g[f"{name}_variables"], m, N, N - n)


def _method(ck, tag):
    return {
        "ms": ck.MinSum(),
        "ms2": ck.MinSum(scale=0.75, offset=0.05, max_iterations=12, early_stop=False),
        "sp0": ck.SumProduct(max_iterations=10, early_stop=False),
        "sp1": ck.SumProduct(max_iterations=10, early_stop=True),
    }[tag]


def _host(res, frames):
    return (res.bits.cpu().numpy().reshape(frames, -1), res.llrs.cpu().numpy().reshape(frames, -1),
            res.valid.cpu().numpy().reshape(-1), res.iterations.cpu().numpy().reshape(-1))  # fmt: skip


def _check_min_sum(g, key, bits, post, valid, iters):
    np.testing.assert_array_equal(iters, g[key + "_iters"], err_msg="iterations")
    np.testing.assert_array_equal(valid, g[key + "_valid"], err_msg="valid")
    np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), g[key + "_bits_packed"],
                                  err_msg="bits")  # fmt: skip
    np.testing.assert_array_equal(post[0], g[key + "_post_first"])
    assert digest(post) == g[key + "_post_digest"]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("tag", TAGS)
def test_reference_decodes(golden_wide, torch_dev, ck, name, tag):
    """Every rule and parameter set of the fixture, default launch."""
    torch, dev = torch_dev
    g = golden_wide
    code = _code(ck, g, name)
    info = code._plan(0).info
    assert info["max_row_degree"] == int(g[f"{name}_max_degree"]) > 27
    assert info["quasi_cyclic"] == (1 if name == "w64qc" else 0)
    llrs = wide_llrs(name, code.n)
    assert digest(llrs) == g[f"{name}_llrs_digest"]
    res = ck.decode(torch.from_numpy(llrs).to(dev), code=code, method=_method(ck, tag))
    bits, post, valid, iters = _host(res, llrs.shape[0])
    key = f"{name}_{tag}"
    if tag.startswith("ms"):
        _check_min_sum(g, key, bits, post, valid, iters)
    else:
        check_sum_product(g, key, bits, post, valid, iters, saturated=True)
    if tag in ("ms", "sp1"):
        assert iters.min() < iters.max()  # early stop: frames end at uneven iterations


@pytest.mark.parametrize("placement", [1, 2])
@pytest.mark.parametrize("threads", [0, 64])
def test_circulant_wide_state_placements(golden_wide, torch_dev, ck, placement, threads):
    """The circulant code with the wide state in shared memory (placement 1)
    and in device memory (2), with one thread per row slot and with half as
    many (two row passes per base row): all bit-identical to the
    reference."""
    torch, dev = torch_dev
    g = golden_wide
    code = _code(ck, g, "w64qc")
    plan = code._plan(0)
    llrs = torch.from_numpy(wide_llrs("w64qc", code.n)).to(dev)
    try:
        plan.set_launch(threads, 0, placement)
        for tag in ("ms", "ms2"):
            res = ck.decode(llrs, code=code, method=_method(ck, tag))
            _check_min_sum(g, f"w64qc_{tag}", *_host(res, llrs.shape[0]))
    finally:
        plan.set_launch(0, 0, 0)


@pytest.mark.parametrize("name", ["w64csr", "dvbs2n910"])
def test_many_frames_against_oracle(golden_wide, torch_dev, ck, name):
    """Many frames of the CSR codes (DVB-S2 normal 9/10 on the plain kernel
    with its posterior in device memory, and on clusters for a small batch)
    against the oracle, bit for bit."""
    torch, dev = torch_dev
    g = golden_wide
    code = _code(ck, g, name)
    frames = 300 if name == "w64csr" else 24
    rng = np.random.default_rng(44)
    mean = rng.uniform(5.0, 10.0, size=(frames, 1))
    llrs = (mean + np.sqrt(2.0 * mean) * rng.standard_normal((frames, code.n))).astype(np.float32)
    method = ck.MinSum(max_iterations=15)
    got = _host(ck.decode(torch.from_numpy(llrs).to(dev), code=code, method=method), frames)
    row_ptr, cols, _ = code._schedule
    want = oracle.decode(llrs, (row_ptr, cols, code.num_variables), k=code.k, max_iterations=15)
    for a, b, what in zip(got, want, ("bits", "llrs", "valid", "iterations"), strict=True):
        np.testing.assert_array_equal(np.asarray(a).reshape(np.shape(b)), b, err_msg=what)
    few = _host(ck.decode(torch.from_numpy(llrs[:3].copy()).to(dev), code=code, method=method), 3)
    for a, b, what in zip(few, got, ("bits", "llrs", "valid", "iterations"), strict=True):
        np.testing.assert_array_equal(a, b[:3], err_msg=f"{what}, 3 frames")


def test_mixed_launch_with_wide_code(golden_wide, torch_dev, ck):
    """A mixed launch of the degree-64 circulant code and code A (the
    any-degree mixed kernel, wide state for both) equals plain decodes."""
    from commkit_gb300 import workloads as W

    torch, dev = torch_dev
    g = golden_wide
    wide = _code(ck, g, "w64qc")
    rng = np.random.default_rng(45)
    mean = rng.uniform(4.0, 10.0, size=(200, 1))
    llr_w = (mean + np.sqrt(2.0 * mean) * rng.standard_normal((200, wide.n))).astype(np.float32)
    spec = W.CODES["A"]
    code_a = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    b = W.coded_batch(spec, 300, 4, 1.5, seed=46)
    llr_a = ck.compute_llr_frames(torch.from_numpy(b.symbols).to(dev), noise_var=b.noise_var,
                                  constellation=ck.Constellation.qam(4))  # fmt: skip
    batches = [(torch.from_numpy(llr_w).to(dev), wide, ck.MinSum(max_iterations=20)),
               (llr_a, code_a, ck.MinSum(max_iterations=20))]  # fmt: skip
    mixed = ck.decode_mixed(batches)
    for (llr, code, method), m in zip(batches, mixed, strict=True):
        p = ck.decode(llr, code=code, method=method)
        frames = m.iterations.shape[0]
        np.testing.assert_array_equal(m.llrs.cpu().numpy(), p.llrs.cpu().numpy().reshape(frames, -1))
        np.testing.assert_array_equal(m.bits.cpu().numpy(), p.bits.cpu().numpy().reshape(frames, -1))
        np.testing.assert_array_equal(m.iterations.cpu().numpy(), p.iterations.cpu().numpy().reshape(-1))
        np.testing.assert_array_equal(m.valid.cpu().numpy(), p.valid.cpu().numpy().reshape(-1))
