"""The per-call extension on the GPU: after a first call through the general
path registers a form, ``decode`` and ``compute_llr`` take the extension,
whose results are bit-identical to the general path's (which the other GPU
tests check against the oracle), with the same shapes, dtypes, result type
and errors; forms it does not take still reach the general path."""

from __future__ import annotations

import dataclasses
import threading

import numpy as np
import pytest

from commkit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import commkit_gb300 as ck
    from commkit_gb300 import _lib

    return torch, torch.device("cuda", 0), ck, _lib


def _llrs(torch, dev, ck, frames, seed, ebn0=2.0):
    b = W.coded_batch(W.CODE_A, frames, 4, ebn0, seed=seed)
    x = torch.from_numpy(b.symbols).to(dev)
    return ck.compute_llr(x, noise_var=float(b.noise_var[0]), constellation=ck.Constellation.qam(4))


def _general(ck, torch, code, llrs, method):
    """``decode`` through the general path: a caller-owned workspace takes it."""
    from commkit_gb300 import coding

    rule = coding._rule_args(coding._resolve_method(method))[0]
    rows = llrs.numel() // code.n
    ws = torch.empty(code._plan(llrs.device.index).workspace_size(rows, rule), dtype=torch.uint8, device=llrs.device)
    return ck.decode(llrs, code=code, method=method, workspace=ws)


def _same_result(a, b):
    for f in ("bits", "llrs", "valid", "iterations"):
        x, y = getattr(a, f), getattr(b, f)
        assert x.dtype == y.dtype and x.shape == y.shape and x.device == y.device, f
        assert bool((x == y).all()), f
    assert a.checked is True and b.checked is True


def test_extension_is_loaded(env):
    torch, dev, ck, _lib = env
    mod = _lib.calls()
    assert mod is not None
    with open("/proc/self/maps") as f:
        assert str(_lib.CALLS_PATH) in f.read()


@pytest.mark.parametrize("shape", ["1d", "1d3", "2d"])
@pytest.mark.parametrize("method", ["default", "minsum", "offset", "sumproduct"])
def test_decode_matches_general_path(env, shape, method):
    torch, dev, ck, _lib = env
    m = {"default": None, "minsum": ck.MinSum(max_iterations=20),
         "offset": ck.MinSum(scale=0.75, offset=0.25, max_iterations=12, early_stop=False),
         "sumproduct": ck.SumProduct(max_iterations=10)}[method]  # fmt: skip
    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    frames = {"1d": 1, "1d3": 3, "2d": 4}[shape]
    llrs = _llrs(torch, dev, ck, frames, seed=5).reshape(-1)
    if shape == "2d":
        llrs = llrs.reshape(2, 2 * code.n)
    first = ck.decode(llrs, code=code, method=m)  # general path; registers the code
    assert code._calls_entries is not None and code._calls_entries[0] is not None
    fast = ck.decode(llrs, code=code, method=m)
    want = _general(ck, torch, code, llrs, m)
    torch.cuda.synchronize()
    _same_result(fast, want)
    _same_result(first, want)
    assert type(fast) is ck.DecodeResult
    with pytest.raises(dataclasses.FrozenInstanceError):
        fast.bits = None


def test_decode_large_outputs_and_kept_parts(env):
    """Outputs above the shared-allocation size are allocated apiece; below
    it they share one, and a part kept alone stays valid."""
    torch, dev, ck, _lib = env
    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    m = ck.MinSum(max_iterations=15)
    big = _llrs(torch, dev, ck, (4 << 20) // (4 * code.n) + 3, seed=6)
    ck.decode(big[:1], code=code, method=m)
    fast = ck.decode(big, code=code, method=m)
    assert fast.llrs.untyped_storage().data_ptr() != fast.bits.untyped_storage().data_ptr()
    _same_result(fast, _general(ck, torch, code, big, m))
    small = big[:2]
    r = ck.decode(small, code=code, method=m)
    assert r.llrs.untyped_storage().data_ptr() == r.bits.untyped_storage().data_ptr()
    bits = r.bits
    del r
    junk = [torch.full((1 << 16,), 7, dtype=torch.uint8, device=dev) for _ in range(8)]
    want = _general(ck, torch, code, small, m)
    torch.cuda.synchronize()
    assert bool((bits == want.bits).all())
    del junk


def test_decode_errors_match(env):
    """A status of the C ABI raises what the general path raises."""
    torch, dev, ck, _lib = env
    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    llrs = _llrs(torch, dev, ck, 1, seed=7)
    ck.decode(llrs, code=code)
    bad = ck.MinSum(max_iterations=2**31)  # -2**31 as the C ABI's int32
    msgs = []
    for _ in range(2):  # the general path, then the extension
        with pytest.raises(ValueError) as e:
            ck.decode(llrs, code=code, method=bad)
        msgs.append(str(e.value))
    assert "_c_call" in bad.__dict__
    assert msgs[0] == msgs[1] and "max_iterations" in msgs[0]


def test_decode_forms_it_declines(env):
    torch, dev, ck, _lib = env
    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    m = ck.MinSum(max_iterations=20)
    llrs = _llrs(torch, dev, ck, 2, seed=8).reshape(2, -1)
    ck.decode(llrs, code=code, method=m)
    want = _general(ck, torch, code, llrs.contiguous(), m)
    strided = torch.empty(2, 2 * code.n, device=dev)[:, ::2]
    strided.copy_(llrs)
    _same_result(ck.decode(strided, code=code, method=m), want)
    with pytest.warns(ck.PrecisionWarning):
        _same_result(ck.decode(llrs.double(), code=code, method=m), want)
    with pytest.raises(ValueError, match="multiple"):
        ck.decode(llrs[:, :-1].contiguous(), code=code, method=m)
    empty = ck.decode(llrs[:0], code=code, method=m)
    assert empty.bits.shape == (0, code.k) and empty.llrs.shape == (0, code.n)


def test_decode_side_stream_and_threads(env):
    torch, dev, ck, _lib = env
    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    m = ck.MinSum(max_iterations=20)
    inputs = [_llrs(torch, dev, ck, 2, seed=20 + i) for i in range(4)]
    wants = [_general(ck, torch, code, x, m) for x in inputs]
    ck.decode(inputs[0], code=code, method=m)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        r = ck.decode(inputs[1], code=code, method=m)
    s.synchronize()
    _same_result(r, wants[1])
    assert (0, s.cuda_stream) in _lib.calls().workspaces()
    torch.cuda.synchronize()
    errors = []

    def worker(i):
        try:
            for _ in range(25):
                got = ck.decode(inputs[i], code=code, method=m)
                torch.cuda.current_stream().synchronize()
                _same_result(got, wants[i])
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors


def _fresh(ck, name):
    """A constellation equal to a factory's but not the factory's cached one,
    so its first call takes the general path."""
    if name == "shaped16":
        c = ck.Constellation.qam(16).shaped(nu=0.1)
    else:
        fam = name.rstrip("0123456789")
        c = getattr(ck.Constellation, fam)(int(name[len(fam):]))
    return ck.Constellation(c.points, c.bit_labels, c.pmf)


@pytest.mark.parametrize("name,method", [("qam16", "maxlog"), ("qam16", "exact"), ("qam64", "exact"),
                                         ("shaped16", "maxlog"), ("psk8", "maxlog"), ("psk8", "exact")])  # fmt: skip
def test_llr_matches_general_path(env, name, method):
    torch, dev, ck, _lib = env
    c = _fresh(ck, name)
    rng = np.random.default_rng(9)
    x = torch.from_numpy((rng.standard_normal((3, 1024)) + 1j * rng.standard_normal((3, 1024))).astype(np.complex64)).to(dev)
    nv = 0.37
    want = ck.compute_llr(x, noise_var=nv, constellation=c, method=method)  # general path; registers
    assert c.__dict__["_calls_llr"][method][0] is not None
    got = ck.compute_llr(x, noise_var=nv, constellation=c, method=method)
    again = c.llr(x, noise_var=nv, method=method)
    for r in (got, again):
        assert r.dtype == want.dtype and r.shape == want.shape == (3, 1024 * c.bits_per_symbol)
        assert bool((r == want).all())
    for v in (np.float64(nv), np.float32(nv), 1):
        w = ck.compute_llr(x, noise_var=float(v), constellation=c, method=method)
        assert bool((ck.compute_llr(x, noise_var=v, constellation=c, method=method) == w).all())
    s = x[0, 5]  # one symbol, a 0-dimensional tensor
    one = ck.compute_llr(s.clone(), noise_var=nv, constellation=c, method=method)
    assert one.shape == (c.bits_per_symbol,)
    assert bool((one == want[0, 5 * c.bits_per_symbol:6 * c.bits_per_symbol]).all())
    strided = ck.compute_llr(x[:, ::2], noise_var=nv, constellation=c, method=method)
    assert bool((strided == want.reshape(3, 1024, -1)[:, ::2].reshape(3, -1)).all())
    for bad in (-1.0, float("nan")):
        with pytest.raises(ValueError, match="noise_var"):
            ck.compute_llr(x, noise_var=bad, constellation=c, method=method)
    with pytest.raises(ValueError, match="Unknown method"):
        ck.compute_llr(x, noise_var=nv, constellation=c, method="max-log")
    torch.cuda.synchronize()
