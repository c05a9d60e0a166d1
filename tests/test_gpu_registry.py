"""The drop-in boundary driven by the reference's own launcher calls.

``registry_calls.npz`` holds the argument tuples that the reference's host
code builds for its CUDA launchers, recorded at its kernel registry while its
``compute_llr`` and ``decode`` ran their GPU route (``make_golden.py
--only=registry``): the closed-form, level-metric and point tables of
``commkit/mapping/_demap.py:184-220, 298-352`` with ``inv_s2`` from
``esn0_db``, and the schedule and zero-padded posterior of
``commkit/coding/ldpc.py:539-588``.  Here ``plugin.install()`` puts this
package's launchers into a registry laid out as ``commkit._cuda``
(``commkit/_cuda/__init__.py:35-81``), each recorded call goes through
``get_kernel(name, **spec)`` with the same arguments on the GPU, and the
results are held to the reference's CPU results on the same input:
max-log LLRs and min-sum decodes bit-exact, exact LLRs within 1e-5 relative
/ 1e-6 absolute, sum-product at the reference's tolerance.
"""

from __future__ import annotations

import types

import numpy as np
import pytest

from tests.conftest import GOLDEN, check_sum_product, digest
from tests.golden.make_golden import REGISTRY_LDPC_CASES, REGISTRY_LLR_CASES, registry_ldpc_llrs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def calls():
    return dict(np.load(GOLDEN / "registry_calls.npz"))


@pytest.fixture(scope="module")
def registry():
    """A module laid out as the reference's registry: ``_KERNEL_FACTORIES``
    and ``get_kernel(name, **spec)`` (``KeyError`` for an unknown name),
    with this package's launchers installed by ``plugin.install``."""
    from commkit_gb300 import plugin

    reg = types.ModuleType("commkit._cuda")
    reg._KERNEL_FACTORIES = {"selftest_scale": object()}

    def get_kernel(name, **spec):
        factory = reg._KERNEL_FACTORIES.get(name)
        if factory is None:
            raise KeyError(f"Unknown CUDA kernel {name!r}; registered: {sorted(reg._KERNEL_FACTORIES)}")
        return factory(**spec)

    reg.get_kernel = get_kernel
    plugin.install(reg)
    yield reg
    plugin.uninstall(reg)


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.device("cuda", 0))


def _kwargs(g, tag):
    out = {}
    for key in g[f"{tag}_kwnames"]:
        v = g[f"{tag}_kw_{key}"]
        out[str(key)] = bool(v) if v.dtype == np.bool_ else (int(v) if v.dtype.kind == "i" else float(v))
    return out


@pytest.mark.parametrize("tag", [c[0] for c in REGISTRY_LLR_CASES])
def test_demapper_launchers_with_reference_calls(calls, registry, tag):
    g = calls
    name = str(g[f"{tag}_name"])
    args = []
    for j in range(int(g[f"{tag}_nargs"])):
        if f"{tag}_arg{j}_len" in g:
            args.append(tuple(_dev(g[f"{tag}_arg{j}_{t}"]) for t in range(int(g[f"{tag}_arg{j}_len"]))))
        else:
            args.append(_dev(g[f"{tag}_arg{j}"]))
    kw = _kwargs(g, tag)
    got = registry.get_kernel(name)(_dev(g[f"{tag}_x"]), *args, **kw).cpu().numpy()
    want = g[f"{tag}_want"]
    assert got.shape == want.shape and got.dtype == np.float32
    if kw.get("exact", False):
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
    else:
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("case", REGISTRY_LDPC_CASES, ids=[c[0] for c in REGISTRY_LDPC_CASES])
def test_ldpc_launcher_with_reference_calls(calls, registry, case):
    """``ldpc_layered`` decodes the reference's posterior in place with its
    own schedule, returning (iterations, valid) as its launcher does."""
    tag, frames, mean = case[0], case[4], case[5]
    g = calls
    n = int(g[f"{tag}_n"])
    app = np.zeros((frames, int(g[f"{tag}_N"])), np.float32)
    app[:, :n] = registry_ldpc_llrs(frames, n, mean)
    assert digest(app) == g[f"{tag}_app_digest"]
    launch = registry.get_kernel(str(g[f"{tag}_name"]), sum_product=bool(g[f"{tag}_sum_product"]))
    a = _dev(app)
    iters, valid = launch(a, _dev(g[f"{tag}_row_ptr"]), _dev(g[f"{tag}_cols"]), _dev(g[f"{tag}_layer_ptr"]),
                          **_kwargs(g, tag))  # fmt: skip
    post = a.cpu().numpy()[:, :n]
    iters, valid = iters.cpu().numpy(), valid.cpu().numpy()
    if bool(g[f"{tag}_sum_product"]):
        bits = (post < 0).astype(np.int8)
        want = {"x_iters": g[f"{tag}_want_iters"], "x_valid": g[f"{tag}_want_valid"], "x_post": g[f"{tag}_want_post"],
                "x_bits_packed": np.packbits((g[f"{tag}_want_post"] < 0).astype(np.uint8), axis=1)}  # fmt: skip
        check_sum_product(want, "x", bits, post, valid, iters, saturated=False)
    else:
        np.testing.assert_array_equal(iters, g[f"{tag}_want_iters"])
        np.testing.assert_array_equal(valid, g[f"{tag}_want_valid"])
        np.testing.assert_array_equal(post[0], g[f"{tag}_want_post_first"])
        assert digest(post) == g[f"{tag}_want_post_digest"]
