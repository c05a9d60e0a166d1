"""Constellations beyond square QAM, on the CPU: the factories against the
reference's points, labels and priors, the routing between the per-axis and
the M-point demappers, and the oracle's LLRs against the reference's own
``Constellation.llr`` (``llr_mpoint_golden.npz``)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300.mapping import Constellation, _table_kind, host_tables, inv_s2
from tests.conftest import GOLDEN

BUILDERS = {
    "psk2": lambda: Constellation.psk(2),
    "psk8": lambda: Constellation.psk(8),
    "psk16": lambda: Constellation.psk(16),
    "qam2": lambda: Constellation.qam(2),
    "qam8": lambda: Constellation.qam(8),
    "qam32": lambda: Constellation.qam(32),
    "qam128": lambda: Constellation.qam(128),
    "qam512": lambda: Constellation.qam(512),
    "pam4": lambda: Constellation.pam(4),
    "pam8u": lambda: Constellation.pam(8, unipolar=True),
    "qam16nu": lambda: Constellation.qam(16).shaped(nu=0.05),
    "qam64h5": lambda: Constellation.qam(64).shaped(entropy=5.0),
    "qam32h4": lambda: Constellation.qam(32).shaped(entropy=4.5),
}


@pytest.fixture(scope="module")
def golden_mpoint():
    return dict(np.load(GOLDEN / "llr_mpoint_golden.npz"))


def build(name: str, g: dict) -> Constellation:
    if name == "custom16":
        return Constellation(g["custom16_points"], g["custom16_bit_labels"], g["custom16_pmf"])
    return BUILDERS[name]()


NAMES = (*BUILDERS, "custom16")


def oracle_llr(c: Constellation, x: np.ndarray, nv: float, method: str) -> np.ndarray:
    """The oracle along the reference's routing: per axis for separable
    lattices, every point otherwise; real symbols count twice the noise."""
    nv = nv if np.iscomplexobj(x) else 2.0 * nv
    exact = method == "exact"
    if c._axes is not None:
        t = host_tables(c, "levels")
        return oracle.llr_levels(x, (t[:4], t[4:]), inv_s2(nv), exact=exact)
    pts, logp, lab = host_tables(c, "points")
    return oracle.llr_points(x, pts, logp, lab, c.bits_per_symbol, inv_s2(nv), exact=exact)


@pytest.mark.parametrize("name", NAMES)
def test_factories_match_reference(golden_mpoint, name):
    g = golden_mpoint
    c = build(name, g)
    np.testing.assert_array_equal(c.points, g[f"{name}_points"])
    np.testing.assert_array_equal(c.bit_labels, g[f"{name}_bit_labels"])
    if g[f"{name}_pmf"].size:
        np.testing.assert_allclose(c.pmf, g[f"{name}_pmf"], rtol=1e-12, atol=1e-15)
    else:
        assert c.pmf is None
    assert c.power() == pytest.approx(float(g[f"{name}_power"]), rel=1e-12)
    assert c.entropy == pytest.approx(float(g[f"{name}_entropy"]), rel=1e-9)
    assert (c._axes is not None) == bool(g[f"{name}_separable"])


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("ni", [0, 1])
def test_oracle_matches_reference_llrs(golden_mpoint, name, ni):
    """Max-log bit for bit; exact within 1e-5 relative / 1e-6 absolute."""
    g = golden_mpoint
    c = build(name, g)
    x = g[f"{name}_x"]
    nv = float(g[f"{name}_n{ni}_nv"])
    np.testing.assert_array_equal(oracle_llr(c, x, nv, "maxlog"), g[f"{name}_n{ni}_maxlog"])
    np.testing.assert_allclose(oracle_llr(c, x, nv, "exact"), g[f"{name}_n{ni}_exact"], rtol=1e-5, atol=1e-6)


def test_routing():
    assert _table_kind(Constellation.qam(64), "maxlog") == "maxlog"
    assert _table_kind(Constellation.qam(64), "exact") == "levels"
    assert _table_kind(Constellation.qam(64).shaped(nu=0.1), "maxlog") == "levels"
    for c in (Constellation.psk(16), Constellation.qam(128), Constellation.qam(8), Constellation.pam(4)):
        assert _table_kind(c, "maxlog") == "points"


def test_constructor_validation():
    with pytest.raises(ValueError, match="power of 2"):
        Constellation(np.arange(6) + 0j)
    with pytest.raises(ValueError, match="distinct"):
        Constellation(np.array([1, 1, 2, 3]) + 0j)
    with pytest.raises(ValueError, match="every bit pattern"):
        Constellation(np.arange(4) + 0j, bit_labels=[[0, 0], [0, 0], [1, 0], [1, 1]])
    with pytest.raises(ValueError, match="sum to 1"):
        Constellation(np.arange(4) + 0j, pmf=[0.5, 0.5, 0.5, 0.5])
    with pytest.raises(ValueError, match="exactly one"):
        Constellation.qam(16).shaped()
    with pytest.raises(ValueError, match="same energy"):
        Constellation.psk(8).shaped(nu=0.1)
    assert Constellation.qam(16) == Constellation.qam(16)
    assert Constellation.qam(16) != Constellation.qam(16).shaped(nu=0.1)
