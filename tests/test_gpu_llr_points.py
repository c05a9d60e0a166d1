"""GPU parity of the M-point demapper and of prior-weighted separable
demapping: sm_103a against the reference's LLRs (``llr_mpoint_golden.npz``)
and the pinned oracle.  Max-log bit for bit; exact within 1e-5 relative /
1e-6 absolute."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300.mapping import Constellation, host_tables, inv_s2
from tests.test_constellations import NAMES, build, oracle_llr

pytestmark = pytest.mark.gpu

TOL = {"rtol": 1e-5, "atol": 1e-6}


@pytest.fixture(scope="module")
def torch_dev():
    import torch

    return torch, torch.device("cuda", 0)


@pytest.fixture(scope="module")
def golden_mpoint():
    from tests.conftest import GOLDEN

    return dict(np.load(GOLDEN / "llr_mpoint_golden.npz"))


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("ni", [0, 1])
def test_compute_llr_matches_reference(golden_mpoint, torch_dev, name, ni):
    """Every constellation through the public API: PSK, 8-QAM, cross QAM,
    real PAM (float32 symbols), shaped square QAM (per-axis priors), shaped
    cross QAM and a random labelled constellation with a prior."""
    import commkit_gb300 as ck

    torch, dev = torch_dev
    g = golden_mpoint
    c = build(name, g)
    x = g[f"{name}_x"]
    nv = float(g[f"{name}_n{ni}_nv"])
    xd = torch.from_numpy(x).to(dev)
    for method in ("maxlog", "exact"):
        got = ck.compute_llr(xd, noise_var=nv, constellation=c, method=method).cpu().numpy()
        got = got.reshape(x.size, -1)
        want = g[f"{name}_n{ni}_{method}"]
        if method == "maxlog":
            np.testing.assert_array_equal(got, want)
        else:
            np.testing.assert_allclose(got, want, **TOL)
            np.testing.assert_allclose(got, oracle_llr(c, x, nv, method), **TOL)


@pytest.mark.parametrize("c", [Constellation.psk(16), Constellation.qam(128), Constellation.qam(32).shaped(entropy=4.5),
                               Constellation.qam(1024).shaped(nu=0.01)], ids=["psk16", "qam128", "qam32h", "qam1024s"])  # fmt: skip
def test_many_symbols_against_oracle(torch_dev, c):
    """2^16 seeded symbols (grid-stride loop, every block)."""
    import commkit_gb300 as ck

    torch, dev = torch_dev
    rng = np.random.default_rng(11)
    n = 1 << 16
    x = (c.points[rng.integers(0, c.order, n)] + 0.1 * (rng.standard_normal(n) + 1j * rng.standard_normal(n)))
    x = x.astype(np.complex64)
    xd = torch.from_numpy(x).to(dev)
    for method in ("maxlog", "exact"):
        got = ck.compute_llr(xd, noise_var=0.05, constellation=c, method=method).cpu().numpy().reshape(n, -1)
        want = oracle_llr(c, x, 0.05, method)
        if method == "maxlog":
            np.testing.assert_array_equal(got, want)
        else:
            np.testing.assert_allclose(got, want, **TOL)


def _raw(torch, dev, x, pts, logp, labels, k, s2, exact):
    from commkit_gb300 import _cuda

    launch = _cuda.get_kernel("llr")
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (x, pts, logp, labels)]
    return launch(*t, k=k, inv_s2=s2, exact=exact).cpu().numpy()


def test_generic_paths_against_oracle(torch_dev):
    """Tables the staged path does not take: labels that are not a
    permutation (repeated), fewer points than labels, and 8192 points
    (13 bits, read from device memory)."""
    torch, dev = torch_dev
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(3000) + 1j * rng.standard_normal(3000)).astype(np.complex64)
    cases = []
    pts = (rng.standard_normal(16) + 1j * rng.standard_normal(16)).astype(np.complex64)
    cases.append((pts, np.zeros(16, np.float32), rng.integers(0, 16, 16).astype(np.int32), 4))
    pts12 = pts[:12].copy()
    cases.append((pts12, rng.uniform(-2, 0, 12).astype(np.float32), rng.permutation(16)[:12].astype(np.int32), 4))
    M = 8192
    big = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    cases.append((big, np.zeros(M, np.float32), rng.permutation(M).astype(np.int32), 13))
    for pts_c, logp, labels, k in cases:
        xs = x[:500] if k == 13 else x
        for exact in (False, True):
            got = _raw(torch, dev, xs, pts_c, logp, labels, k, np.float32(2.5), exact)
            want = oracle.llr_points(xs, pts_c, logp, labels, k, np.float32(2.5), exact=exact)
            if exact:
                np.testing.assert_allclose(got, want, **TOL)
            else:
                np.testing.assert_array_equal(got, want)


def test_launcher_contract(torch_dev):
    """The reference's launcher interface (commkit/_cuda/llr.py:37-84)."""
    torch, dev = torch_dev
    from commkit_gb300 import _cuda

    launch = _cuda.get_kernel("llr")
    c = Constellation.psk(8)
    pts, logp, lab = (torch.from_numpy(a).to(dev) for a in host_tables(c, "points"))
    x = torch.zeros(10, dtype=torch.complex64, device=dev)
    assert launch(x, pts, logp, lab, k=3, inv_s2=1.0, exact=False).shape == (10, 3)
    assert launch(x[:0], pts, logp, lab, k=3, inv_s2=1.0, exact=True).shape == (0, 3)
    with pytest.raises(ValueError, match="bits per symbol"):
        launch(x, pts, logp, lab, k=17, inv_s2=1.0, exact=False)
    with pytest.raises(TypeError, match="complex64"):
        launch(x.to(torch.complex128), pts, logp, lab, k=3, inv_s2=1.0, exact=False)
    with pytest.raises(TypeError, match="int32"):
        launch(x, pts, logp, lab.to(torch.int64), k=3, inv_s2=1.0, exact=False)
    with pytest.raises(ValueError):
        launch(x, pts, logp[:4], lab, k=3, inv_s2=1.0, exact=False)


def test_frames_match_single_calls(torch_dev):
    """One noise variance per frame (ck_llr_points_frames) equals one call
    per frame, for PSK (M-point) and shaped QAM (per-axis priors)."""
    import commkit_gb300 as ck

    torch, dev = torch_dev
    rng = np.random.default_rng(2)
    for c in (Constellation.psk(16), Constellation.qam(64).shaped(entropy=5.0)):
        F, S = 6, 700
        x = (c.points[rng.integers(0, c.order, (F, S))] + 0.2 * rng.standard_normal((F, S))).astype(np.complex64)
        nv = rng.uniform(0.01, 0.3, F)
        xd = torch.from_numpy(x).to(dev)
        for method in ("maxlog", "exact"):
            both = ck.compute_llr_frames(xd, noise_var=nv, constellation=c, method=method).cpu().numpy()
            for f in range(F):
                one = ck.compute_llr(xd[f], noise_var=float(nv[f]), constellation=c, method=method).cpu().numpy()
                np.testing.assert_array_equal(both[f], one)
            np.testing.assert_allclose(both.reshape(F * S, -1)[:S], oracle_llr(c, x[0], float(nv[0]), method),
                                       **TOL)  # fmt: skip
    assert inv_s2(0.0) == np.float32(1e20)
