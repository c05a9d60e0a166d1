"""The continuous-batching server: every request's result is the same as
when it is demapped and decoded alone."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fused,split,spread", [(True, True, False), (True, True, True), (True, False, False),
                                                (False, False, False)])
def test_served_results_equal_standalone_decodes(fused, split, spread):
    import torch

    import commkit_gb300 as ck
    from commkit_gb300 import workloads as W
    from commkit_gb300.serving import PayloadPool, Server, poisson_requests

    dev = torch.device("cuda", 0)
    pool = PayloadPool.build({(n, o): (24 if n == "C" else 64) for n in "ABC" for o in (4, 16, 64)}, seed=1)
    reqs = poisson_requests(3000.0, 0.03, pool, max_frames=20, seed=2)
    assert len(reqs) > 20
    codes = {n: ck.LDPCCode.quasi_cyclic(W.CODES[n].base(), lifting=W.CODES[n].z) for n in "ABC"}
    method = ck.MinSum(max_iterations=30)
    server = Server(codes, method, hbm_budget=2 << 30, max_inflight=3, device=dev, output_arena_bytes=256 << 20,
                    fused=fused, priority_split=split, spread_long=spread)  # fmt: skip
    assert server.fused == fused and server.split == split and server.long_codes == {"C"}
    done = server.serve(reqs)
    assert sorted(r.rid for r in done) == [r.rid for r in reqs]
    assert all(r.latency > 0 for r in done)
    for r in done:
        sym = r.symbols.to(dev)
        llr = ck.compute_llr_frames(sym, noise_var=np.full(r.frames, r.noise_var),
                                    constellation=ck.Constellation.qam(r.order))  # fmt: skip
        alone = ck.decode(llr, code=codes[r.code], method=method)
        np.testing.assert_array_equal(r.bits, alone.bits.cpu().numpy().reshape(r.bits.shape))
        np.testing.assert_array_equal(r.llrs, alone.llrs.cpu().numpy().reshape(r.llrs.shape))
        np.testing.assert_array_equal(r.iterations, alone.iterations.cpu().numpy().reshape(-1))
        np.testing.assert_array_equal(r.valid, alone.valid.cpu().numpy().reshape(-1))
