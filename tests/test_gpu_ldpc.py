"""GPU decoder parity: the sm_103a layered min-sum decoder against the
reference's golden decodes and the pinned CPU oracle, bit for bit
(a-posteriori LLRs, hard decisions, iteration counts, syndrome flags)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300 import workloads as W
from tests.conftest import digest, kat_llrs

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


def _to_np(res, frames):
    return (res.bits.cpu().numpy().reshape(frames, -1), res.llrs.cpu().numpy().reshape(frames, -1),
            res.valid.cpu().numpy().reshape(-1), res.iterations.cpu().numpy().reshape(-1))  # fmt: skip


def _assert_same(got, want):
    for a, b, what in zip(got, want, ("bits", "llrs", "valid", "iterations"), strict=True):
        np.testing.assert_array_equal(a, b, err_msg=what)


def _oracle(code, llrs, **method):
    row_ptr, cols, _ = code._schedule
    return oracle.decode(llrs, (row_ptr, cols, code.num_variables), k=code.k, **method)


@pytest.mark.parametrize("which", ["dvbs2s", "pon"])
@pytest.mark.parametrize("early_stop", [False, True])
def test_reference_kat(golden_ldpc, torch_dev, ck, which, early_stop):
    """The reference's own bit-exactness cases (tests/coding/test_ldpc_kernel.py:24-34):
    DVB-S2 short 1/2 (CSR path) and PON (circulant path, punctured)."""
    torch, dev = torch_dev
    g = golden_ldpc
    m, N, n = (int(g[f"{which}_{s}"]) for s in ("m", "N", "n"))
    code = ck.LDPCCode(g[f"{which}_checks"], g[f"{which}_variables"], m, N, N - n)
    llrs = kat_llrs(n)
    res = ck.decode(torch.from_numpy(llrs).to(dev), code=code,
                    method=ck.MinSum(scale=0.75, offset=0.05, max_iterations=12, early_stop=early_stop))  # fmt: skip
    bits, post, valid, iters = _to_np(res, 6)
    p = f"{which}_es{int(early_stop)}"
    np.testing.assert_array_equal(iters, g[p + "_iters"])
    np.testing.assert_array_equal(valid, g[p + "_valid"])
    np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), g[p + "_bits_packed"])
    np.testing.assert_array_equal(post[0], g[p + "_post_first"])
    assert digest(post) == g[p + "_post_digest"]
    info = code._plan(0).info
    assert info["quasi_cyclic"] == (1 if which == "pon" else 0)


@pytest.mark.parametrize("which", ["dvbs2s", "pon"])
@pytest.mark.parametrize("early_stop", [False, True])
def test_nonfinite_llrs(golden_ldpc, torch_dev, ck, which, early_stop):
    """LLRs with +-inf and a NaN against the reference's decode
    (``ldpc_nonfinite.npz``): a NaN |Q| stays out of min1 and min2 on both
    paths, so every finite result matches bit for bit and NaN sits where
    the reference has NaN."""
    from tests.conftest import GOLDEN

    torch, dev = torch_dev
    g, nf = golden_ldpc, np.load(GOLDEN / "ldpc_nonfinite.npz")
    m, N, n = (int(g[f"{which}_{s}"]) for s in ("m", "N", "n"))
    code = ck.LDPCCode(g[f"{which}_checks"], g[f"{which}_variables"], m, N, N - n)
    res = ck.decode(torch.from_numpy(nf[f"nf_{which}_llrs"]).to(dev), code=code,
                    method=ck.MinSum(max_iterations=12, early_stop=early_stop))  # fmt: skip
    bits, post, valid, iters = _to_np(res, 3)
    p = f"nf_{which}_es{int(early_stop)}"
    np.testing.assert_array_equal(iters, nf[p + "_iters"])
    np.testing.assert_array_equal(valid, nf[p + "_valid"])
    np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), nf[p + "_bits"])
    np.testing.assert_array_equal(post, nf[p + "_post"])


@pytest.mark.parametrize("name,frames,order", [("A", 600, 4), ("B", 400, 16), ("C", 160, 16)])
@pytest.mark.parametrize("placement", [1, 2, 3])
def test_specialised_kernel_equals_table_kernel(torch_dev, ck, name, frames, order, placement):
    """The code-specialised kernel (compiled at run time) against the
    table-driven kernel on the same frames, message state in shared (1;
    code C's does not fit there and stays in device memory) or device (2)
    memory, or one message per edge in shared memory (3: codes A and B; the
    table kernel and code C keep the records): every output bit for bit;
    and against the oracle."""
    from commkit_gb300 import _lib

    torch, dev = torch_dev
    spec = W.CODES[name]
    zp = (spec.z + 31) // 32 * 32
    codes = [_qc_code(ck, name), _qc_code(ck, name)]
    for code, mode in zip(codes, (_lib.CK_LDPC_SPECIALISE_ON, _lib.CK_LDPC_SPECIALISE_OFF), strict=True):
        plan = code._plan(0)
        plan.set_specialise(mode)
        plan.set_launch(zp, 0, placement)
    batch = W.coded_batch(spec, frames, order, W.WATERFALL_DB[name] + 0.5, seed=21)
    x = torch.from_numpy(batch.symbols).to(dev)
    llr = ck.compute_llr_frames(x, constellation=ck.Constellation.qam(order), noise_var=batch.noise_var)
    method = ck.MinSum(max_iterations=30)
    got = [_to_np(ck.decode(llr, code=c, method=method), frames) for c in codes]
    assert codes[0]._plan(0).specialisation()[1] == 1, codes[0]._plan(0).specialisation()
    assert codes[1]._plan(0).specialisation()[1] == 0
    if placement == _lib.CK_LDPC_PLACE_EDGES:
        used = codes[0]._plan(0).resolved_launch()[2], codes[1]._plan(0).resolved_launch()[2]
        assert used == ((3, 1) if name != "C" else (2, 2)), used
    _assert_same(got[0], got[1])
    assert 0 < np.mean(got[0][3]) < 30  # frames stop at different iterations
    _assert_same(got[0], _oracle(codes[0], llr.cpu().numpy(), max_iterations=30))


def test_specialisation_without_nvrtc():
    """Where NVRTC cannot be loaded, AUTO decodes on the table-driven kernel
    (the same bits) and says why, and ON is an error (a child process: the
    library looks for NVRTC once per process)."""
    import os
    import subprocess
    import sys

    code = r"""
import numpy as np, torch, commkit_gb300 as ck
from commkit_gb300 import _lib, workloads as W
s = W.CODES["A"]
code = ck.LDPCCode.quasi_cyclic(s.base(), lifting=s.z)
code._plan(0).set_launch(64, 0, 0)
x = torch.from_numpy((1.0 + np.random.default_rng(0).standard_normal((8, code.n))).astype(np.float32)).cuda()
r = ck.decode(x, code=code)
mode, state, why = code._plan(0).specialisation()
assert state == -1 and "NVRTC not found" in why, (state, why)
code2 = ck.LDPCCode.quasi_cyclic(s.base(), lifting=s.z)
code2._plan(0).set_specialise(_lib.CK_LDPC_SPECIALISE_ON)
code2._plan(0).set_launch(64, 0, 0)
try:
    ck.decode(x, code=code2)
    raise SystemExit("ON without NVRTC did not fail")
except ValueError as e:
    assert "unavailable" in str(e), e
print("ok", int(r.iterations.sum()))
"""
    env = dict(os.environ, COMMKIT_GB300_NVRTC="/nonexistent/libnvrtc.so.13")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = subprocess.run([sys.executable, "-c", code], env=env, cwd=root, capture_output=True, text=True,
                         timeout=300)  # fmt: skip
    assert res.returncode == 0, res.stdout + res.stderr
    assert res.stdout.startswith("ok")


@pytest.mark.parametrize("z,seed", [(27, 1), (32, 2), (100, 3), (160, 4), (45, 5)])
def test_specialised_random_codes(torch_dev, ck, z, seed):
    """Random circulant codes (liftings that are and are not multiples of
    32, rows of degree 2 to 16 over a dual-diagonal parity part, punctured
    columns) decoded by the generated kernel, against the table-driven
    kernel and the oracle."""
    from commkit_gb300 import _lib

    torch, dev = torch_dev
    rng = np.random.default_rng(seed)
    mb, nb = int(rng.integers(3, 9)), int(rng.integers(12, 22))
    base = np.full((mb, nb), -1, dtype=np.int64)
    kb = nb - mb
    for i in range(mb):
        deg = int(rng.integers(1, min(14, kb) + 1))
        cols = rng.choice(kb, size=deg, replace=False)
        base[i, cols] = rng.integers(0, z, size=deg)
        base[i, kb + i] = 0  # dual-diagonal parity part: full rank
        if i + 1 < mb:
            base[i + 1, kb + i] = 0
    punct = z if seed % 2 else 0
    codes = [ck.LDPCCode.quasi_cyclic(base, lifting=z, punctured=punct) for _ in range(2)]
    zp = (z + 31) // 32 * 32
    for code, mode in zip(codes, (_lib.CK_LDPC_SPECIALISE_ON, _lib.CK_LDPC_SPECIALISE_OFF), strict=True):
        code._plan(0).set_specialise(mode)
        code._plan(0).set_launch(zp, 0, 0)
    assert codes[0]._plan(0).info["lifting"] == z
    frames = 96
    llr = (0.8 + 1.6 * rng.standard_normal((frames, codes[0].n))).astype(np.float32)
    x = torch.from_numpy(llr).to(dev)
    method = ck.MinSum(scale=0.8, offset=0.02, max_iterations=15)
    got = [_to_np(ck.decode(x, code=c, method=method), frames) for c in codes]
    assert codes[0]._plan(0).specialisation()[1] == 1
    _assert_same(got[0], got[1])
    _assert_same(got[0], _oracle(codes[0], llr, scale=0.8, offset=0.02, max_iterations=15))


@pytest.mark.parametrize("name", ["A", "B"])
def test_golden_codes(golden_ldpc, torch_dev, ck, name):
    torch, dev = torch_dev
    g = golden_ldpc
    code = _qc_code(ck, name)
    llrs = g[f"{name}_llrs"]
    frames = llrs.shape[0]
    res = ck.decode(torch.from_numpy(llrs).to(dev), code=code,
                    method=ck.MinSum(max_iterations=int(g[f"{name}_max_iterations"])))  # fmt: skip
    bits, post, valid, iters = _to_np(res, frames)
    np.testing.assert_array_equal(iters, g[f"{name}_iters"])
    np.testing.assert_array_equal(valid, g[f"{name}_valid"])
    np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), g[f"{name}_bits_packed"])
    assert digest(post) == g[f"{name}_post_digest"]
    assert code._plan(0).info["lifting"] == W.CODES[name].z


def test_config1_code_a_1024_frames(torch_dev, ck):
    """Config 1: code A, QPSK at Eb/N0 2.5 dB, exact LLRs, MinSum(max_iterations=20),
    1024 frames: the GPU demap + decode against the oracle, frame for frame."""
    torch, dev = torch_dev
    code = _qc_code(ck, "A")
    batch = W.coded_batch(W.CODE_A, 1024, 4, 2.5, seed=1)
    x = torch.from_numpy(batch.symbols).to(dev)
    c = ck.Constellation.qam(4)
    llr = ck.compute_llr(x, noise_var=float(batch.noise_var[0]), constellation=c, method="exact")
    llr_np = llr.cpu().numpy()
    want_llr = oracle.llr(batch.symbols.reshape(-1), 4, oracle.inv_s2(batch.noise_var[0]),
                          method="exact").reshape(1024, -1)  # fmt: skip
    np.testing.assert_allclose(llr_np, want_llr, rtol=1e-5, atol=1e-6)
    method = ck.MinSum(max_iterations=20)
    res = ck.decode(llr, code=code, method=method)
    got = _to_np(res, 1024)
    _assert_same(got, _oracle(code, llr_np, max_iterations=20))
    # FER against the transmitted bits is then identical too; report it.
    fer = np.mean(np.any(got[0] != batch.info, axis=1))
    assert fer < 0.5


@pytest.mark.parametrize("frames", [96])
def test_config3_code_c(torch_dev, ck, frames):
    """Config 3 (code C, 16-QAM max-log at Eb/N0 1.0 dB, 50 iterations) on a
    slice of frames: max-log LLRs and the decode both bit-exact."""
    torch, dev = torch_dev
    code = _qc_code(ck, "C")
    batch = W.coded_batch(W.CODE_C, frames, 16, 1.0, seed=1)
    x = torch.from_numpy(batch.symbols).to(dev)
    llr = ck.compute_llr(x, noise_var=float(batch.noise_var[0]), constellation=ck.Constellation.qam(16))
    llr_np = llr.cpu().numpy()
    want = oracle.llr(batch.symbols.reshape(-1), 16, oracle.inv_s2(batch.noise_var[0])).reshape(frames, -1)
    np.testing.assert_array_equal(llr_np, want)
    res = ck.decode(llr, code=code, method=ck.MinSum(max_iterations=50))
    _assert_same(_to_np(res, frames), _oracle(code, llr_np, max_iterations=50))


@pytest.mark.parametrize("name", ["A", "C"])
def test_launch_shapes_do_not_change_results(torch_dev, ck, name):
    """Every launch shape (threads per frame, frames per block, message
    placement) gives the same bits: the autotuner only changes speed."""
    torch, dev = torch_dev
    code = _qc_code(ck, name)
    spec = W.CODES[name]
    order = 4 if name == "A" else 16
    frames = 40
    batch = W.coded_batch(spec, frames, order, 2.0 if name == "A" else 2.5, seed=4)
    x = torch.from_numpy(batch.symbols).to(dev)
    llr = ck.compute_llr(x, noise_var=float(batch.noise_var[0]), constellation=ck.Constellation.qam(order))
    method = ck.MinSum(max_iterations=12)
    plan = code._plan(0)
    base = _to_np(ck.decode(llr, code=code, method=method), frames)
    _assert_same(base, _oracle(code, llr.cpu().numpy(), max_iterations=12))
    shapes = [(32, 1, 0), (32, 3, 0), (64, 2, 1), (128, 1, 2), (256, 2, 0), (512, 1, 2), (64, 0, 3), (384, 1, 3)]
    try:
        for T, G, place in shapes:
            try:
                plan.set_launch(T, G, place)
                ws = plan.workspace_size(frames)
            except ValueError:
                continue  # shape does not fit this code
            assert ws > 0
            got = _to_np(ck.decode(llr, code=code, method=method), frames)
            _assert_same(got, base)
    finally:
        plan.set_launch(0, 0, 0)


def test_noiseless_codewords_stop_before_the_first_iteration(torch_dev, ck):
    """``tests/coding/test_ldpc.py:157-165``: codewords decode with 0 iterations."""
    torch, dev = torch_dev
    code = _qc_code(ck, "A")
    info = np.random.default_rng(2).integers(0, 2, (5, code.k), dtype=np.int8)
    words = W.encode_qc(W.CODE_A.base(), 54, info)
    res = ck.decode(torch.from_numpy(words).to(dev), code=code)  # int input: hard decisions
    bits, _, valid, iters = _to_np(res, 5)
    np.testing.assert_array_equal(bits, info)
    assert valid.all() and (iters == 0).all()


def test_random_llrs_fail_with_max_iterations(torch_dev, ck):
    """``tests/coding/test_ldpc.py:254-262``: noise decodes to invalid after max_iterations."""
    torch, dev = torch_dev
    code = _qc_code(ck, "B")
    llrs = np.random.default_rng(5).standard_normal((3, code.n)).astype(np.float32)
    res = ck.decode(torch.from_numpy(llrs).to(dev), code=code, method=ck.MinSum(max_iterations=4))
    _, _, valid, iters = _to_np(res, 3)
    assert not valid.any() and (iters == 4).all()
    res = ck.decode(torch.from_numpy(llrs).to(dev), code=code,
                    method=ck.MinSum(max_iterations=3, early_stop=False))  # fmt: skip
    assert (res.iterations.cpu().numpy() == 3).all()


def test_inplace_launcher_and_contract(torch_dev, ck):
    """The reference's launcher interface (commkit/_cuda/coding.py:27-67):
    in-place ``app``, (iters, valid) back, dtype/shape errors, B = 0."""
    torch, dev = torch_dev
    from commkit_gb300 import _cuda

    code = _qc_code(ck, "A")
    row_ptr, cols, layer_ptr = (torch.from_numpy(a.copy()).to(dev) for a in code._schedule)
    launch = _cuda.get_kernel("ldpc_layered")
    llrs = (1.0 + 1.5 * np.random.default_rng(3).standard_normal((7, code.num_variables))).astype(np.float32)
    app = torch.from_numpy(llrs).to(dev)
    kw = dict(scale=0.875, offset=0.0, max_iterations=9, early_stop=True)
    iters, valid = launch(app, row_ptr, cols, layer_ptr, **kw)
    row, col, _ = code._schedule
    post, want_it, want_ok = oracle.ldpc_layered(llrs.copy(), row, col, max_iterations=9)
    np.testing.assert_array_equal(app.cpu().numpy(), post)
    np.testing.assert_array_equal(iters.cpu().numpy(), want_it)
    np.testing.assert_array_equal(valid.cpu().numpy(), want_ok)
    with pytest.raises(TypeError, match="float32"):
        launch(app.to(torch.float64), row_ptr, cols, layer_ptr, **kw)
    with pytest.raises(TypeError, match="int32"):
        launch(app, row_ptr.to(torch.int64), cols, layer_ptr, **kw)
    it0, ok0 = launch(app[:0], row_ptr, cols, layer_ptr, **kw)
    assert it0.shape == (0,) and ok0.shape == (0,)


def test_decode_shapes_and_errors(torch_dev, ck):
    torch, dev = torch_dev
    code = _qc_code(ck, "A")
    x = torch.zeros((2, 3 * code.n), dtype=torch.float32, device=dev)
    res = ck.decode(x, code=code)
    assert res.bits.shape == (2, 3 * code.k) and res.llrs.shape == (2, 3 * code.n)
    assert res.valid.shape == (2, 3) and res.iterations.shape == (2, 3) and res.checked
    assert res.valid.dtype == torch.bool
    res1 = ck.decode(x[0], code=code)
    assert res1.bits.shape == (3 * code.k,)
    with pytest.raises(ValueError, match="multiple"):
        ck.decode(x[:, :-1], code=code)
    with pytest.raises(TypeError, match="method"):
        ck.decode(x, code=code, method="min-sum")
    with pytest.warns(ck.PrecisionWarning):
        ck.decode(x.to(torch.float64), code=code)
    empty = ck.decode(x[:0], code=code)
    assert empty.bits.shape == (0, 3 * code.k)


def test_workspace_is_reused_and_status_is_clean(torch_dev, ck):
    torch, dev = torch_dev
    from commkit_gb300 import _device, _lib

    code = _qc_code(ck, "C")
    batch = W.coded_batch(W.CODE_C, 6, 16, 3.0, seed=9)
    llr = ck.compute_llr(torch.from_numpy(batch.symbols).to(dev), noise_var=float(batch.noise_var[0]),
                         constellation=ck.Constellation.qam(16))  # fmt: skip
    plan = code._plan(0)
    ws = torch.empty(plan.workspace_size(6), dtype=torch.uint8, device=dev)
    a = _to_np(ck.decode(llr, code=code, workspace=ws), 6)
    b = _to_np(ck.decode(llr, code=code, workspace=ws), 6)
    _assert_same(a, b)
    st = _lib.lib().ck_ldpc_workspace_status(_device.wrap(ws).ptr, _device.stream_of(_device.wrap(ws)))
    assert st == _lib.CK_OK


def test_dvbs2_normal_frames(torch_dev, ck):
    """DVB-S2 normal-frame rate 1/2 (N = 64800, CSR rows, posterior in
    device memory): the reference's decode of two QPSK frames at Es/N0
    1.5 dB bit for bit, and 64 codewords (its benchmark's batch) against the
    oracle."""
    from commkit_gb300.workloads import awgn, encode_accumulate, map_bits
    from tests.conftest import GOLDEN
    from tests.golden.make_golden import dvbs2_symbols

    torch, dev = torch_dev
    d = dict(np.load(GOLDEN / "dvbs2_normal.npz"))
    m, N, n, k = (int(d[f"dvbs2n_{s}"]) for s in ("m", "N", "n", "k"))
    code = ck.LDPCCode(d["dvbs2n_checks"], d["dvbs2n_variables"], m, N, N - n)
    assert code._plan(0).info["quasi_cyclic"] == 0
    words = np.unpackbits(d["dvbs2n_words"], axis=1)[:, :n].astype(np.int8)
    rx, nv = dvbs2_symbols(words[:2], 1.5, seed=5)
    c = ck.Constellation.qam(4)
    llr = ck.compute_llr(torch.from_numpy(rx).to(dev), noise_var=nv, constellation=c)
    assert digest(llr.cpu().numpy()) == d["dvbs2n_llrs_digest"]
    res = ck.decode(llr, code=code)
    bits, post, valid, iters = _to_np(res, 2)
    np.testing.assert_array_equal(iters, d["dvbs2n_iters"])
    np.testing.assert_array_equal(valid, d["dvbs2n_valid"])
    np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), d["dvbs2n_bits_packed"])
    assert digest(post) == d["dvbs2n_post_digest"]

    rng = np.random.default_rng(12)
    info = rng.integers(0, 2, size=(64, k), dtype=np.int8)
    sym = awgn(map_bits(encode_accumulate(d["dvbs2n_checks"], d["dvbs2n_variables"], m, k, info), 4), nv, rng)
    llr = ck.compute_llr(torch.from_numpy(sym).to(dev), noise_var=nv, constellation=c).reshape(64, n)
    got = _to_np(ck.decode(llr, code=code), 64)
    _assert_same(got, _oracle(code, llr.cpu().numpy(), max_iterations=50))


@pytest.mark.parametrize("rule, early_stop", [("min_sum", True), ("min_sum", False), ("sum_product", True)])
def test_cluster_decode_equals_plain(torch_dev, ck, rule, early_stop):
    """DVB-S2 normal frames: a small batch runs on thread-block clusters (one
    frame per cluster of CTAs, the posterior in device memory), a large one
    on the plain persistent kernel; the same frames decode identically."""
    from commkit_gb300.workloads import awgn, encode_accumulate, map_bits
    from tests.conftest import GOLDEN

    torch, dev = torch_dev
    d = dict(np.load(GOLDEN / "dvbs2_normal.npz"))
    m, N, n, k = (int(d[f"dvbs2n_{s}"]) for s in ("m", "N", "n", "k"))
    code = ck.LDPCCode(d["dvbs2n_checks"], d["dvbs2n_variables"], m, N, N - n)
    rng = np.random.default_rng(17)
    frames = 400
    info = rng.integers(0, 2, size=(frames, k), dtype=np.int8)
    nv = 10.0 ** (-1.2 / 10.0)
    sym = awgn(map_bits(encode_accumulate(d["dvbs2n_checks"], d["dvbs2n_variables"], m, k, info), 4), nv, rng)
    llr = ck.compute_llr(torch.from_numpy(sym).to(dev), noise_var=nv, constellation=ck.Constellation.qam(4))
    llr = llr.reshape(frames, n)
    method = (ck.MinSum(max_iterations=15, early_stop=early_stop) if rule == "min_sum"
              else ck.SumProduct(max_iterations=8, early_stop=early_stop))  # fmt: skip
    big = _to_np(ck.decode(llr, code=code, method=method), frames)
    for few in (3, 40):
        small = _to_np(ck.decode(llr[:few].contiguous(), code=code, method=method), few)
        for a, b, what in zip(small, big, ("bits", "llrs", "valid", "iterations"), strict=True):
            np.testing.assert_array_equal(a, b[:few], err_msg=f"{what}, {few} frames")
    if rule == "min_sum":
        row_ptr, cols, _ = code._schedule
        want = oracle.decode(llr[:3].cpu().numpy(), (row_ptr, cols, N), k=k, max_iterations=15,
                             early_stop=early_stop)  # fmt: skip
        _assert_same(_to_np(ck.decode(llr[:3].contiguous(), code=code, method=method), 3), want)
