"""The continuous feed (``ck_ldpc_feed_launch``, ``serving.FeedServer``): one
persistent decoder takes frames that the host publishes into pinned rings
while it runs.  Every request's results equal its standalone demap and
decode and the oracle's, bit for bit; a decoder that has returned for lack
of work is launched again and continues where it stopped; the stop flag
ends it at once."""

from __future__ import annotations

import time

import numpy as np
import pytest

import oracle
from commkit_gb300 import workloads as W

# A feed that stopped delivering would leave serve() polling: fail the test instead.
pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300)]


def _codes(ck):
    return {n: ck.LDPCCode.quasi_cyclic(W.CODES[n].base(), lifting=W.CODES[n].z) for n in "ABC"}


def _check_standalone(ck, codes, method, done, dev):
    for r in done:
        llr = ck.compute_llr_frames(r.symbols.to(dev), noise_var=np.full(r.frames, r.noise_var),
                                    constellation=ck.Constellation.qam(r.order))  # fmt: skip
        alone = ck.decode(llr, code=codes[r.code], method=method)
        np.testing.assert_array_equal(r.bits, alone.bits.cpu().numpy().reshape(r.bits.shape))
        np.testing.assert_array_equal(r.llrs, alone.llrs.cpu().numpy().reshape(r.llrs.shape))
        np.testing.assert_array_equal(r.iterations, alone.iterations.cpu().numpy().reshape(-1))
        np.testing.assert_array_equal(r.valid, alone.valid.cpu().numpy().reshape(-1))


@pytest.mark.parametrize("policy", ["oldest", "short_first"])
def test_feed_results_equal_standalone_decodes(policy):
    """A Poisson stream of every code and constellation through the feed,
    under either queue policy."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.serving import FeedServer, PayloadPool, poisson_requests

    dev = torch.device("cuda", 0)
    pool = PayloadPool.build({(n, o): (24 if n == "C" else 64) for n in "ABC" for o in (4, 16, 64)}, seed=1)
    reqs = poisson_requests(3000.0, 0.03, pool, max_frames=20, seed=2)
    assert len(reqs) > 20
    codes = _codes(ck)
    method = ck.MinSum(max_iterations=30)
    server = FeedServer(codes, method, device=dev, ring_frames=1 << 10, output_arena_bytes=256 << 20,
                        idle_us=5000, policy=policy, max_inflight_frames=256)  # fmt: skip
    done = server.serve(reqs)
    assert sorted(r.rid for r in done) == [r.rid for r in reqs]
    assert all(r.latency > 0 for r in done)
    _check_standalone(ck, codes, method, done, dev)
    server.close()


def test_feed_against_oracle_with_ring_wrap():
    """A ring of 64 frames per queue, so positions wrap several times, and
    every frame checked against the oracle on its own symbols."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.serving import FeedServer, PayloadPool, poisson_requests

    dev = torch.device("cuda", 0)
    pool = PayloadPool.build({(n, o): (16 if n == "C" else 48) for n in "ABC" for o in (4, 16, 64)}, seed=4)
    reqs = poisson_requests(4000.0, 0.05, pool, max_frames=12, seed=5)
    codes = _codes(ck)
    method = ck.MinSum(max_iterations=50)
    server = FeedServer(codes, method, device=dev, ring_frames=64, output_arena_bytes=128 << 20, idle_us=5000)
    done = server.serve(reqs)
    assert sorted(r.rid for r in done) == [r.rid for r in reqs]
    per_queue = {}
    for r in done:
        per_queue[(r.code, r.order)] = per_queue.get((r.code, r.order), 0) + r.frames
    assert max(per_queue.values()) > 64  # some queue's ring wrapped
    seen = set()
    for r in done:
        sym = r.symbols.cpu().numpy().reshape(r.frames, -1)
        llrs = np.stack([oracle.llr(sym[f], r.order, oracle.inv_s2(r.noise_var)).reshape(-1)
                         for f in range(r.frames)])  # fmt: skip
        row, col, _ = codes[r.code]._schedule
        bits, post, valid, iters = oracle.decode(llrs, (row, col, codes[r.code].num_variables), k=codes[r.code].k,
                                                 max_iterations=50)  # fmt: skip
        np.testing.assert_array_equal(r.bits.reshape(bits.shape), bits)
        np.testing.assert_array_equal(r.llrs.reshape(post.shape), post)
        np.testing.assert_array_equal(r.valid.reshape(-1), valid)
        np.testing.assert_array_equal(r.iterations.reshape(-1), iters)
        seen.add(r.code)
    assert seen == {"A", "B", "C"}
    server.close()


def test_feed_relaunches_after_idle_and_stops_on_request():
    """With a 1 ms idle limit, requests 30 ms apart each find the decoder
    gone and launch it again (continuing from the counts in its workspace);
    the stop flag then ends a decoder that would otherwise wait 1 s."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300.serving import FeedServer, PayloadPool, Request

    dev = torch.device("cuda", 0)
    pool = PayloadPool.build({("A", 4): 32, ("B", 16): 32}, seed=6)
    codes = _codes(ck)
    method = ck.MinSum(max_iterations=20)
    server = FeedServer({n: codes[n] for n in "AB"}, method, device=dev, orders=(4, 16), ring_frames=256,
                        output_arena_bytes=64 << 20, idle_us=1000)  # fmt: skip
    reqs = []
    for i in range(4):
        name, order = ("A", 4) if i % 2 == 0 else ("B", 16)
        sym, nv = pool.frames[(name, order)]
        reqs.append(Request(i, name, order, sym[4 * i : 4 * i + 4], float(nv[4 * i]), arrival=0.03 * i))
    done = server.serve(reqs)
    assert sorted(r.rid for r in done) == [0, 1, 2, 3]
    assert server.launches == 4
    _check_standalone(ck, codes, method, done, dev)
    # A decoder that would wait a second for work returns at once when asked.
    server.idle_us = 1_000_000
    sym, nv = pool.frames[("A", 4)]
    done = server.serve([Request(9, "A", 4, sym[:3], float(nv[0]))])
    assert len(done) == 1
    t0 = time.perf_counter()
    server.close()
    assert time.perf_counter() - t0 < 0.5
    assert server.event.query()
    _check_standalone(ck, codes, method, done, dev)
