"""GPU demapper parity: the sm_103a kernels against the reference's golden
LLRs and the pinned CPU oracle.  Max-log is bit-exact; exact (log-sum-exp)
agrees within rtol 1e-5, atol 1e-6."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6


@pytest.fixture(scope="module")
def torch_dev():
    import torch

    return torch, torch.device("cuda", 0)


@pytest.fixture(scope="module")
def ck():
    import commkit_gb300

    return commkit_gb300


@pytest.mark.parametrize("order", [4, 16, 64, 256])
@pytest.mark.parametrize("ni", [0, 1, 2])
def test_golden_vectors(golden_llr, torch_dev, ck, order, ni):
    torch, dev = torch_dev
    key = f"q{order}_n{ni}"
    x = torch.from_numpy(golden_llr[key + "_x"]).to(dev)
    nv = float(golden_llr[key + "_nv"])
    c = ck.Constellation.qam(order)
    k = c.bits_per_symbol
    got = ck.compute_llr(x, noise_var=nv, constellation=c, method="maxlog").cpu().numpy()
    np.testing.assert_array_equal(got.reshape(-1, k), golden_llr[key + "_closed"])
    got = ck.compute_llr(x, noise_var=nv, constellation=c, method="exact").cpu().numpy()
    np.testing.assert_allclose(got.reshape(-1, k), golden_llr[key + "_exact"], rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("order", [16, 64])
@pytest.mark.parametrize("method", ["maxlog", "exact"])
def test_demapper_at_scale_per_frame_noise(torch_dev, ck, order, method):
    """Config 2 at full size: 2^22 symbols in 1024 frames of 4096 with
    per-frame Es/N0 in [8, 20] dB, one batched launch, against the oracle."""
    torch, dev = torch_dev
    rx, nv = W.demapper_batch(order, frames=1024, frame_len=4096, seed=3)
    x = torch.from_numpy(rx).to(dev)
    c = ck.Constellation.qam(order)
    got = ck.compute_llr_frames(x, noise_var=nv, constellation=c, method=method).cpu().numpy()
    s2 = (1.0 / np.maximum(nv, 1e-20)).astype(np.float32)
    want = oracle.llr(rx.reshape(-1), order, s2, method=method, frame_len=4096).reshape(1024, -1)
    if method == "maxlog":
        np.testing.assert_array_equal(got, want)
    else:
        np.testing.assert_allclose(got, want, rtol=RTOL, atol=ATOL)
    # the batched form equals one plain call per frame
    for f in (0, 511, 1023):
        one = ck.compute_llr(x[f], noise_var=float(nv[f]), constellation=c, method=method)
        np.testing.assert_array_equal(one.cpu().numpy(), got[f])


@pytest.mark.parametrize("method", ["maxlog", "exact"])
def test_odd_sizes_and_unaligned_buffers(torch_dev, ck, method):
    torch, dev = torch_dev
    rng = np.random.default_rng(5)
    rx = (rng.standard_normal(4099) + 1j * rng.standard_normal(4099)).astype(np.complex64)
    c = ck.Constellation.qam(64)
    x = torch.from_numpy(rx).to(dev)
    for lo, hi in ((0, 4099), (1, 4099), (1, 4098), (0, 1), (3, 4)):
        view = x[lo:hi]  # offset views are 8- but not 16-byte aligned
        got = ck.compute_llr(view, noise_var=0.07, constellation=c, method=method).cpu().numpy()
        want = oracle.llr(rx[lo:hi], 64, oracle.inv_s2(0.07), method=method).reshape(-1)
        if method == "maxlog":
            np.testing.assert_array_equal(got, want)
        else:
            np.testing.assert_allclose(got, want, rtol=RTOL, atol=ATOL)


def test_shapes_empty_and_errors(torch_dev, ck):
    torch, dev = torch_dev
    c = ck.Constellation.qam(16)
    x = torch.zeros((3, 5), dtype=torch.complex64, device=dev)
    assert ck.compute_llr(x, noise_var=0.1, constellation=c).shape == (3, 20)
    assert ck.compute_llr(x[:, :0], noise_var=0.1, constellation=c).shape == (3, 0)
    with pytest.raises(ValueError, match="one of"):
        ck.compute_llr(x, constellation=c)
    with pytest.raises(ValueError, match="Unknown method"):
        ck.compute_llr(x, noise_var=0.1, constellation=c, method="map")
    # complex128 is reduced to float32 with a warning
    with pytest.warns(ck.PrecisionWarning):
        ck.compute_llr(x.to(torch.complex128), noise_var=0.1, constellation=c)


def test_launchers_follow_the_reference_contract(torch_dev, ck):
    """The registry's launchers: dtype -> TypeError, shape -> ValueError."""
    torch, dev = torch_dev
    from commkit_gb300 import _cuda
    from commkit_gb300.mapping import device_tables
    from commkit_gb300 import _device

    c = ck.Constellation.qam(16)
    x = torch.zeros(8, dtype=torch.complex64, device=dev)
    tabs = device_tables(c, "maxlog", _device.wrap(x))
    launch = _cuda.get_kernel("llr_separable_maxlog")
    out = launch(x, tabs[:5], tabs[5:], inv_s2=10.0)
    assert out.shape == (8, 4) and out.dtype == torch.float32
    with pytest.raises(TypeError, match="complex64"):
        launch(x.to(torch.complex128), tabs[:5], tabs[5:], inv_s2=10.0)
    with pytest.raises(ValueError, match="shape"):
        launch(x.reshape(2, 4), tabs[:5], tabs[5:], inv_s2=10.0)
    with pytest.raises(TypeError, match="int32"):
        launch(x, (tabs[0], tabs[1].to(torch.int64), *tabs[2:5]), tabs[5:], inv_s2=10.0)
    with pytest.raises(KeyError):
        _cuda.get_kernel("no_such_kernel")
    lv = device_tables(c, "levels", _device.wrap(x))
    out2 = _cuda.get_kernel("llr_separable")(x, lv[:4], lv[4:], inv_s2=10.0, exact=False)
    np.testing.assert_array_equal(out2.cpu().numpy(), out.cpu().numpy())
