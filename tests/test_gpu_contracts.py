"""The reference's API rules for this path (``tests/test_api_contracts.py``):
calls leave their inputs unchanged, return arrays on the input's device with
the input's rank, and reject host and foreign arrays with ``TypeError``."""

from __future__ import annotations

import numpy as np
import pytest

from commkit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch

    import commkit_gb300 as ck

    dev = torch.device("cuda", 0)
    spec = W.CODES["A"]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    batch = W.coded_batch(spec, 6, 4, 2.0, seed=3)
    return torch, ck, dev, code, batch


def test_no_mutation_device_and_rank(setup):
    torch, ck, dev, code, batch = setup
    c = ck.Constellation.qam(4)
    x = torch.from_numpy(batch.symbols).to(dev)
    x0 = x.clone()
    llr = ck.compute_llr(x, noise_var=float(batch.noise_var[0]), constellation=c)
    assert torch.equal(x, x0) and llr.device == x.device and llr.ndim == x.ndim
    l0 = llr.clone()
    res = ck.decode(llr, code=code, method=ck.MinSum(max_iterations=20))
    assert torch.equal(llr, l0)
    for t in (res.bits, res.llrs, res.valid, res.iterations):
        assert t.device == llr.device and t.ndim == llr.ndim
    one = ck.decode(llr[0], code=code)
    assert one.bits.ndim == 1 and one.valid.shape == (1,)
    bits = torch.from_numpy(batch.info.astype(np.int8)).to(dev)
    b0 = bits.clone()
    words = ck.encode(bits, code=code)
    assert torch.equal(bits, b0) and words.device == bits.device and words.ndim == bits.ndim
    sent = words.to(torch.int8)
    s0 = sent.clone()
    g = ck.gmi(llr, sent, constellation=c)
    assert torch.equal(sent, s0) and torch.equal(llr, l0) and g.shape == (6,)


def test_host_and_foreign_arrays_are_rejected(setup):
    torch, ck, dev, code, batch = setup
    c = ck.Constellation.qam(4)
    for bad in (batch.symbols, torch.from_numpy(batch.symbols), [1.0, 2.0]):
        with pytest.raises(TypeError):
            ck.compute_llr(bad, noise_var=0.1, constellation=c)
    with pytest.raises(TypeError):
        ck.decode(np.zeros((2, code.n), np.float32), code=code)
    with pytest.raises(TypeError):
        ck.encode(np.zeros((2, code.k), np.int8), code=code)


def test_gmi_rejects_noise_arguments_for_llr_arrays(setup):
    torch, ck, dev, code, batch = setup
    c = ck.Constellation.qam(4)
    llr = torch.zeros((2, 8), dtype=torch.float32, device=dev)
    bits = torch.zeros((2, 8), dtype=torch.int8, device=dev)
    for kw in ({"noise_var": 0.1}, {"esn0_db": 3.0}):
        with pytest.raises(ValueError, match="Signal input"):
            ck.gmi(llr, bits, constellation=c, **kw)
        with pytest.raises(ValueError, match="Signal input"):
            ck.ngmi(llr, bits, constellation=c, **kw)
