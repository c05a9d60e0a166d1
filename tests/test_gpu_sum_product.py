"""GPU sum-product parity: the sm_103a layered sum-product decoder against
the reference's CPU decodes (``ldpc_sp_golden.npz``) and the pinned CPU
oracle.  Hard decisions, syndrome flags and iteration counts must match
exactly; posteriors at the reference's own GPU-vs-CPU tolerance (see
``check_sum_product``)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300 import workloads as W
from tests.conftest import SP_SATURATED, SP_TAGS, check_sum_product

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_dev():
    import torch

    return torch, torch.device("cuda", 0)


@pytest.fixture(scope="module")
def ck():
    import commkit_gb300

    return commkit_gb300


def _qc_code(ck, name):
    spec = W.CODES[name]
    return ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)


def _host(res, frames):
    return (res.bits.cpu().numpy().reshape(frames, -1), res.llrs.cpu().numpy().reshape(frames, -1),
            res.valid.cpu().numpy().reshape(-1), res.iterations.cpu().numpy().reshape(-1))  # fmt: skip


@pytest.mark.parametrize("tag", SP_TAGS)
@pytest.mark.parametrize("early_stop", [False, True])
def test_reference_cases(golden_ldpc, golden_sp, torch_dev, ck, tag, early_stop):
    """The reference's own sum-product case (DVB-S2 short 1/2, CSR rows) and
    PON (circulant rows, message state in device memory), low and high SNR."""
    torch, dev = torch_dev
    g, sp = golden_ldpc, golden_sp
    which = str(sp[f"sp_{tag}_code"])
    m, N, n = (int(g[f"{which}_{s}"]) for s in ("m", "N", "n"))
    code = ck.LDPCCode(g[f"{which}_checks"], g[f"{which}_variables"], m, N, N - n)
    llrs = sp[f"sp_{tag}_llrs"]
    method = ck.SumProduct(max_iterations=int(sp[f"sp_{tag}_max_iterations"]), early_stop=early_stop)
    res = ck.decode(torch.from_numpy(llrs).to(dev), code=code, method=method)
    bits, post, valid, iters = _host(res, llrs.shape[0])
    check_sum_product(sp, f"sp_{tag}_es{int(early_stop)}", bits, post, valid, iters,
                      saturated=tag in SP_SATURATED)  # fmt: skip
    assert code._plan(0).info["quasi_cyclic"] == (1 if which == "pon" else 0)


@pytest.mark.parametrize("name, frames, order, ebn0, its",
                         [("A", 96, 4, 1.2, 12), ("B", 64, 16, 5.0, 10), ("C", 3, 16, 4.5, 6)])  # fmt: skip
def test_seeded_codes_against_oracle(torch_dev, ck, name, frames, order, ebn0, its):
    """Circulant rows of the seeded codes near their waterfalls, with early
    stop: codes A and B keep the per-edge messages in shared memory, code C
    in device memory.  Frames converge at uneven iterations, so posteriors
    are held to the saturated-case bound."""
    torch, dev = torch_dev
    spec = W.CODES[name]
    code = _qc_code(ck, name)
    batch = W.coded_batch(spec, frames, order, ebn0, seed=31)
    llr = ck.compute_llr(torch.from_numpy(batch.symbols).to(dev), noise_var=float(batch.noise_var[0]),
                         constellation=ck.Constellation.qam(order), method="maxlog")  # fmt: skip
    llr = llr.reshape(frames, code.n)
    res = ck.decode(llr, code=code, method=ck.SumProduct(max_iterations=its))
    bits, post, valid, iters = _host(res, frames)
    row_ptr, cols, _ = code._schedule
    w_bits, w_post, w_valid, w_iters = oracle.decode(llr.cpu().numpy(), (row_ptr, cols, code.num_variables),
                                                     k=code.k, sum_product=True, max_iterations=its)  # fmt: skip
    want = {"x_iters": w_iters, "x_valid": w_valid, "x_post": w_post,
            "x_bits_packed": np.packbits(w_bits.astype(np.uint8), axis=1)}  # fmt: skip
    check_sum_product(want, "x", bits, post, valid, iters, saturated=True)
    assert 0 < valid.sum() < frames or name == "C"  # a mix of converged and failed frames


@pytest.mark.parametrize("name", ["A", "B"])
def test_launch_shapes_do_not_change_results(torch_dev, ck, name):
    """Each row's arithmetic is fixed, so threads per frame change nothing."""
    torch, dev = torch_dev
    code = _qc_code(ck, name)
    rng = np.random.default_rng(5)
    llr = torch.from_numpy((1.0 + 2.0 * rng.standard_normal((40, code.n))).astype(np.float32)).to(dev)
    method = ck.SumProduct(max_iterations=6)
    plan = code._plan(0)
    zp = (W.CODES[name].z + 31) // 32 * 32
    outs = []
    try:
        for t in sorted({32, zp, 2 * zp} if zp % 32 == 0 and 2 * zp <= 512 else {zp}):
            plan.set_launch(t, 0, 0)
            outs.append(_host(ck.decode(llr, code=code, method=method), 40))
    finally:
        plan.set_launch(0, 0, 0)
    for other in outs[1:]:
        for a, b in zip(outs[0], other, strict=True):
            np.testing.assert_array_equal(a, b)


def test_inplace_launcher(torch_dev, ck):
    """``get_kernel("ldpc_layered", sum_product=True)`` decodes ``app`` in
    place, as the reference's launcher does (commkit/_cuda/coding.py:11-67)."""
    torch, dev = torch_dev
    from commkit_gb300 import _cuda

    code = _qc_code(ck, "A")
    row_ptr, cols, layer_ptr = (torch.from_numpy(a.copy()).to(dev) for a in code._schedule)
    launch = _cuda.get_kernel("ldpc_layered", sum_product=True)
    llrs = (1.0 + 1.5 * np.random.default_rng(3).standard_normal((7, code.num_variables))).astype(np.float32)
    app = torch.from_numpy(llrs).to(dev)
    iters, valid = launch(app, row_ptr, cols, layer_ptr, scale=1.0, offset=0.0, max_iterations=9,
                          early_stop=True)  # fmt: skip
    res = ck.decode(torch.from_numpy(llrs).to(dev), code=code, method=ck.SumProduct(max_iterations=9))
    np.testing.assert_array_equal(app.cpu().numpy(), res.llrs.cpu().numpy())
    np.testing.assert_array_equal(iters.cpu().numpy(), res.iterations.cpu().numpy().reshape(-1))
    np.testing.assert_array_equal(valid.cpu().numpy(), res.valid.cpu().numpy().reshape(-1))


def test_mixed_launch_rejects_sum_product(torch_dev, ck):
    torch, dev = torch_dev
    code = _qc_code(ck, "A")
    x = torch.zeros((2, code.n), dtype=torch.float32, device=dev)
    with pytest.raises(NotImplementedError):
        ck.decode_mixed([(x, code, ck.SumProduct())])


@pytest.mark.parametrize("scale,offset", [(0.0, 0.0), (1.5, 0.0), (float("nan"), 0.0), (0.875, -0.1),
                                          (0.875, float("inf"))])
def test_min_sum_launcher_rejects_parameters_minsum_refuses(torch_dev, ck, scale, offset):
    """The C ABI takes the min-sum parameters the reference's MinSum accepts
    (commkit/coding/ldpc.py:345-347: scale in (0, 1], offset finite and
    >= 0) and raises ValueError through the launcher for the others, before
    any launch; ``app`` is left as it was."""
    torch, dev = torch_dev
    from commkit_gb300 import _cuda

    code = _qc_code(ck, "A")
    row_ptr, cols, layer_ptr = (torch.from_numpy(a.copy()).to(dev) for a in code._schedule)
    launch = _cuda.get_kernel("ldpc_layered")
    llrs = np.ones((2, code.num_variables), dtype=np.float32)
    app = torch.from_numpy(llrs).to(dev)
    with pytest.raises(ValueError, match="scale|offset"):
        launch(app, row_ptr, cols, layer_ptr, scale=scale, offset=offset, max_iterations=5, early_stop=True)
    np.testing.assert_array_equal(app.cpu().numpy(), llrs)
