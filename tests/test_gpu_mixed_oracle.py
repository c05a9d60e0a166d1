"""The batched and served forms against the oracle directly (not through the
plain CUDA path): sampled frames of every code from ``decode_mixed``, from
the mixed receiver (fused demapping or not, device or pinned host buffers),
from the full-size config-4 batch (8192 frames, 16 sampled per code) and
from the request server, each demapped and decoded by the oracle on the
same symbols.  Max-log LLRs, posteriors, hard decisions, flags and
iteration counts are bit-exact."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _code(ck, name):
    return ck.LDPCCode.quasi_cyclic(W.CODES[name].base(), lifting=W.CODES[name].z)


def _oracle_frames(code, symbols, noise_var, order, max_iterations):
    """Oracle demap (max-log, each frame's own noise) and decode of frames."""
    llrs = np.stack([oracle.llr(symbols[f], order, oracle.inv_s2(noise_var[f])).reshape(-1)
                     for f in range(symbols.shape[0])])  # fmt: skip
    row, col, _ = code._schedule
    bits, post, valid, iters = oracle.decode(llrs, (row, col, code.num_variables), k=code.k,
                                             max_iterations=max_iterations)  # fmt: skip
    return llrs, bits, post, valid, iters


def _assert_frames(res, idx, want, what):
    _, bits, post, valid, iters = want
    np.testing.assert_array_equal(res.bits.cpu().numpy()[idx], bits, err_msg=f"{what}: bits")
    np.testing.assert_array_equal(res.llrs.cpu().numpy()[idx], post, err_msg=f"{what}: posteriors")
    np.testing.assert_array_equal(res.valid.cpu().numpy().reshape(-1)[idx], valid, err_msg=f"{what}: valid")
    np.testing.assert_array_equal(res.iterations.cpu().numpy().reshape(-1)[idx], iters,
                                  err_msg=f"{what}: iterations")  # fmt: skip


def test_decode_mixed_against_oracle():
    import torch

    import commkit_gb300 as ck

    dev = torch.device("cuda", 0)
    work = W.mixed_workload(total=900, seed=31)
    method = ck.MinSum(max_iterations=50)
    batches, meta = [], []
    for n, b in work.items():
        code = _code(ck, n)
        order = W.MIXED_ORDERS[n]
        llr = ck.compute_llr_frames(torch.from_numpy(b.symbols).to(dev), noise_var=b.noise_var,
                                    constellation=ck.Constellation.qam(order))  # fmt: skip
        batches.append((llr, code, method))
        meta.append((n, code, b, order))
    results = ck.decode_mixed(batches)
    for (n, code, b, order), r in zip(meta, results, strict=True):
        idx = np.linspace(0, b.symbols.shape[0] - 1, 16).astype(int)
        want = _oracle_frames(code, b.symbols[idx], b.noise_var[idx], order, 50)
        _assert_frames(r, idx, want, f"code {n}")


@pytest.mark.parametrize("fused,host_io", [(True, False), (True, True), (False, False)])
def test_receiver_against_oracle(fused, host_io):
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.pipeline import CodeSlot, MixedReceiver

    dev = torch.device("cuda", 0)
    work = W.mixed_workload(total=600, seed=32)
    method = ck.MinSum(max_iterations=50)
    names = list(work)
    codes = {n: _code(ck, n) for n in names}
    slots = [CodeSlot(codes[n], ck.Constellation.qam(W.MIXED_ORDERS[n]), work[n].symbols.shape[0], method)
             for n in names]  # fmt: skip
    rx = MixedReceiver(slots, dev, host_io=host_io, fused=fused)
    rx.load([work[n].symbols for n in names], [work[n].noise_var for n in names])
    rx.step()
    torch.cuda.synchronize()
    for r, n in zip(rx.results(), names, strict=True):
        b = work[n]
        idx = np.linspace(0, b.symbols.shape[0] - 1, 16).astype(int)
        want = _oracle_frames(codes[n], b.symbols[idx], b.noise_var[idx], W.MIXED_ORDERS[n], 50)
        _assert_frames(r, idx, want, f"code {n}")


def test_full_size_mixed_batch_against_oracle():
    """Config 4 at full size, as the benchmark runs it: 8192 frames of codes
    A/B/C (60/30/10) through the fused receiver in one launch; 16 frames of
    every code against the oracle."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.pipeline import CodeSlot, MixedReceiver

    dev = torch.device("cuda", 0)
    work = W.mixed_workload(total=8192, seed=33)
    method = ck.MinSum(max_iterations=50)
    names = list(work)
    assert sum(work[n].symbols.shape[0] for n in names) == 8192
    codes = {n: _code(ck, n) for n in names}
    slots = [CodeSlot(codes[n], ck.Constellation.qam(W.MIXED_ORDERS[n]), work[n].symbols.shape[0], method)
             for n in names]  # fmt: skip
    rx = MixedReceiver(slots, dev, fused=True)
    rx.load([work[n].symbols for n in names], [work[n].noise_var for n in names])
    rx.step()
    torch.cuda.synchronize()
    for r, n in zip(rx.results(), names, strict=True):
        b = work[n]
        idx = np.linspace(0, b.symbols.shape[0] - 1, 16).astype(int)
        want = _oracle_frames(codes[n], b.symbols[idx], b.noise_var[idx], W.MIXED_ORDERS[n], 50)
        _assert_frames(r, idx, want, f"code {n}")
        its = r.iterations.cpu().numpy()
        assert its.min() < its.max()


def test_served_requests_against_oracle():
    """Requests of every code and constellation through the server (fused
    demapping, priority split), each checked frame by frame against the
    oracle on its own symbols and Es/N0."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.serving import PayloadPool, Server, poisson_requests

    dev = torch.device("cuda", 0)
    pool = PayloadPool.build({(n, o): (16 if n == "C" else 48) for n in "ABC" for o in (4, 16, 64)}, seed=4)
    reqs = poisson_requests(2000.0, 0.03, pool, max_frames=12, seed=5)
    codes = {n: _code(ck, n) for n in "ABC"}
    method = ck.MinSum(max_iterations=50)
    server = Server(codes, method, hbm_budget=2 << 30, max_inflight=3, device=dev, output_arena_bytes=256 << 20)
    done = server.serve(reqs)
    assert sorted(r.rid for r in done) == [r.rid for r in reqs]
    seen = set()
    for r in done:
        sym = r.symbols.cpu().numpy().reshape(r.frames, -1)
        want = _oracle_frames(codes[r.code], sym, np.full(r.frames, r.noise_var), r.order, 50)
        _, bits, post, valid, iters = want
        np.testing.assert_array_equal(r.bits.reshape(bits.shape), bits)
        np.testing.assert_array_equal(r.llrs.reshape(post.shape), post)
        np.testing.assert_array_equal(r.valid.reshape(-1), valid)
        np.testing.assert_array_equal(r.iterations.reshape(-1), iters)
        seen.add((r.code, r.order))
    assert {c for c, _ in seen} == {"A", "B", "C"}
