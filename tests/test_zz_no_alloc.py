"""The allocation-free decoder entry point, ``ck_ldpc_decode_static``.

For callers that cannot allocate device memory while they decode (a
real-time receive loop, a fixed start-up memory budget, a host runtime that
owns the device memory), the library decodes with scratch from a static
device array instead of a workspace.  These tests call it through the C ABI
and check that two calls in a row give exactly what ``ck_ldpc_decode``
gives.  This file sorts last so a failure here leaves every other test run.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from commkit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _decode_c_abi(lib, plan, llr, n, k, method, *, static, ws=None, rule=0):
    import torch

    from commkit_gb300 import _device, _lib

    B = llr.shape[0]
    out = torch.empty_like(llr)
    bits = torch.empty((B, k), dtype=torch.int8, device=llr.device)
    iters = torch.empty(B, dtype=torch.int32, device=llr.device)
    valid = torch.empty(B, dtype=torch.uint8, device=llr.device)
    stream = torch.cuda.current_stream(llr.device).cuda_stream
    common = (plan.handle, llr.data_ptr(), out.data_ptr(), B, n, rule,
              float(np.float32(method[0])), float(np.float32(method[1])), method[2], 1,
              iters.data_ptr(), valid.data_ptr(), bits.data_ptr(), k)  # fmt: skip
    if static:
        st = lib.ck_ldpc_decode_static(*common, stream)
    else:
        st = lib.ck_ldpc_decode(*common, _device.wrap(ws).ptr, ws.numel(), stream)
    _lib.check(st, "decode")
    torch.cuda.synchronize()
    return out.cpu().numpy(), bits.cpu().numpy(), iters.cpu().numpy(), valid.cpu().numpy()


@pytest.mark.parametrize("name, frames, order, ebn0", [("C", 700, 16, 1.8), ("A", 300, 4, 2.0)])
def test_static_scratch_matches_workspace_decode(name, frames, order, ebn0):
    """Code C keeps its message state in device memory (the static array
    is used in full, 700 frames > one wave of slots); code A keeps it in
    shared memory (only the header is used)."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300 import _lib

    dev = torch.device("cuda", 0)
    spec = W.CODES[name]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    batch = W.coded_batch(spec, frames, order, ebn0, seed=21)
    llr = ck.compute_llr(torch.from_numpy(batch.symbols).to(dev), noise_var=float(batch.noise_var[0]),
                         constellation=ck.Constellation.qam(order))  # fmt: skip
    plan = code._plan(0)
    plan.set_launch(0, 0, 0)
    ws = torch.empty(plan.workspace_size(frames), dtype=torch.uint8, device=dev)
    lib = _lib.lib()
    method = (0.875, 0.0, 30)
    want = _decode_c_abi(lib, plan, llr, code.n, code.k, method, static=False, ws=ws)
    for _ in range(2):  # two calls in a row share and reuse the static array
        got = _decode_c_abi(lib, plan, llr, code.n, code.k, method, static=True)
        for a, b in zip(got, want, strict=True):
            np.testing.assert_array_equal(a, b)
    assert (want[2] > 0).any()


def test_static_scratch_sum_product():
    """Sum-product through the static scratch: code C's per-edge messages
    (480 KB a frame) in the static array, fewer slots than frames."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300 import _lib

    dev = torch.device("cuda", 0)
    spec = W.CODES["C"]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    rng = np.random.default_rng(8)
    llr = torch.from_numpy((1.5 + 2.0 * rng.standard_normal((200, code.n))).astype(np.float32)).to(dev)
    plan = code._plan(0)
    ws = torch.empty(plan.workspace_size(200, _lib.CK_LDPC_SUM_PRODUCT), dtype=torch.uint8, device=dev)
    lib = _lib.lib()
    method = (1.0, 0.0, 4)
    sp = _lib.CK_LDPC_SUM_PRODUCT
    want = _decode_c_abi(lib, plan, llr, code.n, code.k, method, static=False, ws=ws, rule=sp)
    for _ in range(2):
        got = _decode_c_abi(lib, plan, llr, code.n, code.k, method, static=True, rule=sp)
        for a, b in zip(got, want, strict=True):
            np.testing.assert_array_equal(a, b)
