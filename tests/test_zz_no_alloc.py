"""The allocation-free decoder entry point, ``ck_ldpc_decode_static``.

For callers that cannot allocate device memory while they decode (a
real-time receive loop, a fixed start-up memory budget, a host runtime that
owns the device memory), the library decodes with scratch from a static
device array instead of a workspace.  These tests call it through the C ABI
and check that two calls in a row give exactly what ``ck_ldpc_decode``
gives, that the calls leave the device's free memory unchanged, and that
the first call on a fresh plan compiles nothing.  This file sorts last so a
failure here leaves every other test run.
"""

from __future__ import annotations

import numpy as np
import pytest

from commkit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


class _Call:
    """Output buffers of one decode, allocated once, and the C-ABI call that
    fills them (the static entry point, or ck_ldpc_decode with a workspace)."""

    def __init__(self, plan, llr, n, k, method, rule=0):
        import torch

        B = llr.shape[0]
        self.plan, self.llr, self.n, self.k, self.rule, self.method = plan, llr, n, k, rule, method
        self.out = torch.empty_like(llr)
        self.bits = torch.empty((B, k), dtype=torch.int8, device=llr.device)
        self.iters = torch.empty(B, dtype=torch.int32, device=llr.device)
        self.valid = torch.empty(B, dtype=torch.uint8, device=llr.device)
        self.stream = torch.cuda.current_stream(llr.device).cuda_stream

    def _args(self):
        m = self.method
        return (self.plan.handle, self.llr.data_ptr(), self.out.data_ptr(), self.llr.shape[0], self.n,
                self.rule, float(np.float32(m[0])), float(np.float32(m[1])), m[2], 1,
                self.iters.data_ptr(), self.valid.data_ptr(), self.bits.data_ptr(), self.k)  # fmt: skip

    def static(self):
        from commkit_gb300 import _lib

        _lib.check(_lib.lib().ck_ldpc_decode_static(*self._args(), self.stream), "ck_ldpc_decode_static")

    def workspace(self, ws):
        from commkit_gb300 import _device, _lib

        st = _lib.lib().ck_ldpc_decode(*self._args(), _device.wrap(ws).ptr, ws.numel(), self.stream)
        _lib.check(st, "ck_ldpc_decode")

    def result(self):
        import torch

        torch.cuda.synchronize()
        return (self.out.cpu().numpy(), self.bits.cpu().numpy(), self.iters.cpu().numpy(),
                self.valid.cpu().numpy())  # fmt: skip


def _assert_same(got, want):
    for a, b in zip(got, want, strict=True):
        np.testing.assert_array_equal(a, b)


def _free_bytes():
    import torch

    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


@pytest.mark.parametrize("name, frames, order, ebn0", [("C", 700, 16, 1.8), ("A", 300, 4, 2.0)])
def test_static_scratch_matches_workspace_decode(name, frames, order, ebn0):
    """Code C keeps its min-sum state in device memory (212 KB a frame slot:
    its full grid of slots, 64 MB, fits in the 64 MiB array, and 700 frames
    run through them); code A keeps it in shared memory (only the array's
    header is used).  Two calls in a row equal the workspace decode, and
    after the first call (the set-up) the calls change the device's free
    memory by nothing."""
    import torch

    import commkit_gb300 as ck

    dev = torch.device("cuda", 0)
    spec = W.CODES[name]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    batch = W.coded_batch(spec, frames, order, ebn0, seed=21)
    llr = ck.compute_llr(torch.from_numpy(batch.symbols).to(dev), noise_var=float(batch.noise_var[0]),
                         constellation=ck.Constellation.qam(order))  # fmt: skip
    plan = code._plan(0)
    plan.set_launch(0, 0, 0)
    ws = torch.empty(plan.workspace_size(frames), dtype=torch.uint8, device=dev)
    method = (0.875, 0.0, 30)
    ref = _Call(plan, llr, code.n, code.k, method)
    ref.workspace(ws)
    want = ref.result()
    call = _Call(plan, llr, code.n, code.k, method)
    call.static()  # first call on this device: looks up the array's address
    _assert_same(call.result(), want)
    before = _free_bytes()
    for _ in range(2):  # two calls in a row share and reuse the static array
        call.static()
        _assert_same(call.result(), want)
    assert _free_bytes() == before
    assert (want[2] > 0).any()


def test_static_scratch_sum_product():
    """Sum-product through the static scratch: code C's per-edge messages
    (446 KB a frame) in the static array, which holds fewer frame slots than
    the full grid has, so the grid is cut (the workspace of the uncut grid
    is larger than the array)."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300 import _lib

    dev = torch.device("cuda", 0)
    spec = W.CODES["C"]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    rng = np.random.default_rng(8)
    llr = torch.from_numpy((1.5 + 2.0 * rng.standard_normal((200, code.n))).astype(np.float32)).to(dev)
    plan = code._plan(0)
    sp = _lib.CK_LDPC_SUM_PRODUCT
    ws_bytes = plan.workspace_size(200, sp)
    assert ws_bytes > _lib.CK_LDPC_STATIC_SCRATCH_BYTES
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    method = (1.0, 0.0, 4)
    ref = _Call(plan, llr, code.n, code.k, method, rule=sp)
    ref.workspace(ws)
    want = ref.result()
    call = _Call(plan, llr, code.n, code.k, method, rule=sp)
    before = _free_bytes()
    for _ in range(2):
        call.static()
        _assert_same(call.result(), want)
    assert _free_bytes() == before


def test_static_first_call_on_fresh_plan_compiles_nothing():
    """On a fresh plan the static entry point runs the table-driven kernel
    (it never compiles the code-specialised one, which would load a module)
    and leaves the plan's specialisation untried; after a workspace decode
    has compiled it, the static call runs it.  All results are identical."""
    import torch

    import commkit_gb300 as ck

    dev = torch.device("cuda", 0)
    spec = W.CODES["B"]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    batch = W.coded_batch(spec, 200, 16, 5.0, seed=23)
    llr = ck.compute_llr(torch.from_numpy(batch.symbols).to(dev), noise_var=float(batch.noise_var[0]),
                         constellation=ck.Constellation.qam(16))  # fmt: skip
    plan = code._plan(0)
    method = (0.875, 0.0, 20)
    first = _Call(plan, llr, code.n, code.k, method)
    first.static()
    got_first = first.result()
    assert plan.specialisation()[1] == 0  # nothing compiled
    ws = torch.empty(plan.workspace_size(200), dtype=torch.uint8, device=dev)
    ref = _Call(plan, llr, code.n, code.k, method)
    ref.workspace(ws)
    want = ref.result()
    _assert_same(got_first, want)
    again = _Call(plan, llr, code.n, code.k, method)
    again.static()
    _assert_same(again.result(), want)
