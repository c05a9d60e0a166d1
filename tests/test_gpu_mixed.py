"""The mixed-code persistent launch: frames of codes A, B and C in one
kernel launch give exactly the results of one plain call per code."""

from __future__ import annotations

import numpy as np
import pytest

from commkit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _batch(ck, dev, name, frames, order, ebn0, seed):
    import torch

    spec = W.CODES[name]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    b = W.coded_batch(spec, frames, order, ebn0, seed=seed)
    x = torch.from_numpy(b.symbols).to(dev)
    llr = ck.compute_llr_frames(x, noise_var=b.noise_var, constellation=ck.Constellation.qam(order))
    return code, llr


@pytest.mark.parametrize("placement", [0, 2, 3])
@pytest.mark.parametrize("specialise,parts", [("table_plain", 1), ("both_auto", 1), ("both_auto", 2)])
def test_mixed_launch_matches_plain_calls(placement, specialise, parts):
    """table_plain: plain calls on the table-driven kernel, the mixed launch
    on the code-specialised one (compiled at run time); both_auto: both
    specialised; parts 2: the mixed launch with two threads per row slot."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300 import _lib

    dev = torch.device("cuda", 0)
    cases = [("A", 700, 4, 1.5, ck.MinSum(max_iterations=20)),
             ("B", 300, 16, 5.0, ck.MinSum(scale=0.75, offset=0.05, max_iterations=30)),
             ("C", 90, 16, 2.5, ck.MinSum(max_iterations=50, early_stop=True))]  # fmt: skip
    batches, plain = [], []
    for i, (name, frames, order, ebn0, method) in enumerate(cases):
        code, llr = _batch(ck, dev, name, frames, order, ebn0, seed=30 + i)
        code._plan(0).set_launch(0, 0, placement)
        if specialise == "table_plain":
            code._plan(0).set_specialise(_lib.CK_LDPC_SPECIALISE_OFF)
        batches.append((llr, code, method))
        plain.append(ck.decode(llr, code=code, method=method))
        code._plan(0).set_specialise(_lib.CK_LDPC_SPECIALISE_AUTO)
        if parts == 2:
            code._plan(0).set_launch(2 * ((code._plan(0).info["lifting"] + 31) // 32 * 32), 0, placement)
    mixed = ck.decode_mixed(batches)
    for (llr, code, method), p, m in zip(batches, plain, mixed, strict=True):
        frames = llr.shape[0]
        np.testing.assert_array_equal(m.llrs.cpu().numpy(), p.llrs.cpu().numpy().reshape(frames, -1))
        np.testing.assert_array_equal(m.bits.cpu().numpy(), p.bits.cpu().numpy().reshape(frames, -1))
        np.testing.assert_array_equal(m.iterations.cpu().numpy(), p.iterations.cpu().numpy().reshape(-1))
        np.testing.assert_array_equal(m.valid.cpu().numpy(), p.valid.cpu().numpy().reshape(-1))
        code._plan(0).set_launch(0, 0, 0)
    its = np.concatenate([m.iterations.cpu().numpy() for m in mixed])
    assert its.min() < its.max()  # uneven iteration counts across the launch


def test_mixed_single_code_and_empty_batch():
    import torch

    import commkit_gb300 as ck

    dev = torch.device("cuda", 0)
    code, llr = _batch(ck, dev, "B", 50, 16, 4.0, seed=3)
    method = ck.MinSum(max_iterations=10)
    [m] = ck.decode_mixed([(llr, code, method)])
    p = ck.decode(llr, code=code, method=method)
    np.testing.assert_array_equal(m.llrs.cpu().numpy(), p.llrs.cpu().numpy())
    m0, m1 = ck.decode_mixed([(llr[:0], code, method), (llr, code, method)])
    assert m0.bits.shape == (0, code.k)
    np.testing.assert_array_equal(m1.bits.cpu().numpy(), p.bits.cpu().numpy())


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("host_io", [False, True])
def test_receiver_graph_replay_matches_plain_calls(host_io, fused):
    """The mixed receiver, captured once as a CUDA graph and replayed on a
    new batch, gives the plain calls' results; with ``host_io`` its kernels
    read the symbols from and write the results to pinned host memory, and
    ``fused`` demaps inside the decoder (the same LLR bits)."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.pipeline import CodeSlot, MixedReceiver

    dev = torch.device("cuda", 0)
    work = W.mixed_workload(total=600, seed=5)
    method = ck.MinSum(max_iterations=40)
    names = list(work)
    codes = {n: ck.LDPCCode.quasi_cyclic(W.CODES[n].base(), lifting=W.CODES[n].z) for n in names}
    consts = {n: ck.Constellation.qam(W.MIXED_ORDERS[n]) for n in names}
    rx = MixedReceiver([CodeSlot(codes[n], consts[n], work[n].symbols.shape[0], method) for n in names], dev,
                       host_io=host_io, fused=fused)  # fmt: skip
    assert rx.sym[0].is_cuda != host_io and rx.outputs[0][0].is_cuda != host_io
    assert rx.fused == [fused] * len(names)
    rx.load([work[n].symbols for n in names], [work[n].noise_var for n in names])
    rx.capture()
    work2 = W.mixed_workload(total=600, seed=6)  # same shapes, new frames
    rx.load([work2[n].symbols for n in names], [work2[n].noise_var for n in names])
    rx.run()
    torch.cuda.synchronize()
    for r, n in zip(rx.results(), names, strict=True):
        llr = ck.compute_llr_frames(torch.from_numpy(work2[n].symbols).to(dev), noise_var=work2[n].noise_var,
                                    constellation=consts[n])  # fmt: skip
        p = ck.decode(llr, code=codes[n], method=method)
        np.testing.assert_array_equal(r.llrs.cpu().numpy(), p.llrs.cpu().numpy())
        np.testing.assert_array_equal(r.bits.cpu().numpy(), p.bits.cpu().numpy())
        np.testing.assert_array_equal(r.iterations.cpu().numpy(), p.iterations.cpu().numpy().reshape(-1))


@pytest.mark.parametrize("order", [4, 16, 64, 256])
def test_fused_demap_every_square_order(order):
    """The decoder's fused demapping against the demapper kernel, one to four
    bits per axis, on noisy symbols plus ties at level midpoints, far-out
    points and non-finite coordinates; an exact-LLR slot beside it is
    demapped by the demapper kernel first."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.pipeline import CodeSlot, MixedReceiver

    dev = torch.device("cuda", 0)
    code = ck.LDPCCode.quasi_cyclic(W.CODES["B"].base(), lifting=W.CODES["B"].z)
    c = ck.Constellation.qam(order)
    k = c.bits_per_symbol
    S = code.n // k
    F = 7
    rng = np.random.default_rng(order)
    pts = c.points.astype(np.complex64)
    sym = pts[rng.integers(0, order, size=(F, S))] + (0.15 * (rng.standard_normal((F, S))
                                                             + 1j * rng.standard_normal((F, S)))).astype(np.complex64)
    sym = sym.astype(np.complex64)
    lev = np.unique(pts.real)
    mid = (lev[:-1] + lev[1:]) / 2
    sym[0, : mid.size] = (mid + 1j * mid[::-1]).astype(np.complex64)  # ties
    sym[1, :4] = np.array([50 + 50j, -50 - 50j, np.inf + 0j, complex(np.nan, 1.0)], np.complex64)
    nv = np.linspace(0.05, 0.4, F)
    method = ck.MinSum(max_iterations=8)
    slots = [CodeSlot(code, c, F, method), CodeSlot(code, c, F, method, demap="exact")]
    rx = MixedReceiver(slots, dev, fused=True)
    assert rx.fused == [True, False]
    rx.load([sym, sym], [nv, nv])
    rx.step()
    torch.cuda.synchronize()
    x = torch.from_numpy(sym).to(dev)
    for r, how in zip(rx.results(), ("maxlog", "exact"), strict=True):
        llr = ck.compute_llr_frames(x, noise_var=nv, constellation=c, method=how)
        p = ck.decode(llr, code=code, method=method)
        np.testing.assert_array_equal(r.llrs.cpu().numpy(), p.llrs.cpu().numpy())
        np.testing.assert_array_equal(r.iterations.cpu().numpy(), p.iterations.cpu().numpy().reshape(-1))
