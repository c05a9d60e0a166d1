"""The CPU oracle against the golden fixtures produced by the reference itself.

Pins every oracle function (and the product's host-side tables) to the
reference's outputs on the same inputs; the GPU parity tests then compare
the CUDA path with this pinned oracle.  CPU only.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from commkit_gb300 import workloads as W
from commkit_gb300.mapping import Constellation, host_tables
from tests.conftest import SP_SATURATED, SP_TAGS, check_sum_product, digest, kat_llrs

ORDERS = (4, 16, 64, 256)


@pytest.mark.parametrize("order", ORDERS)
def test_qam_points_and_tables(golden_qam, order):
    g = golden_qam
    np.testing.assert_array_equal(W.gray_qam_points(order), g[f"q{order}_points"])
    np.testing.assert_array_equal(oracle.gray_qam_points(order), g[f"q{order}_points"])
    axes = oracle.qam_axes(order)
    prod = host_tables(Constellation.qam(order), "maxlog")
    for i, name in enumerate(("re", "im")):
        levels, labels, pos = axes[i]
        lo, hi = oracle.opposite_levels(labels)
        np.testing.assert_array_equal(levels.astype(np.float32), g[f"q{order}_{name}_levels"])
        np.testing.assert_array_equal(oracle.packed(labels), g[f"q{order}_{name}_labels"])
        np.testing.assert_array_equal(lo, g[f"q{order}_{name}_lo"])
        np.testing.assert_array_equal(hi, g[f"q{order}_{name}_hi"])
        np.testing.assert_array_equal(pos, g[f"q{order}_{name}_pos"])
        # the product's tables (commkit_gb300.mapping) are the same arrays
        for got, key in zip(prod[5 * i : 5 * i + 5], ("levels", "labels", "lo", "hi", "pos"), strict=True):
            np.testing.assert_array_equal(got, g[f"q{order}_{name}_{key}"])
    assert Constellation.qam(order).power() == pytest.approx(float(g[f"q{order}_power"]), rel=1e-15)


@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("ni", [0, 1, 2])
def test_llr_oracle_matches_reference(golden_llr, order, ni):
    g = golden_llr
    key = f"q{order}_n{ni}"
    x = g[key + "_x"]
    s2 = g[key + "_inv_s2"]
    assert np.float32(1.0 / float(g[key + "_nv"])) == s2 == oracle.inv_s2(float(g[key + "_nv"]))
    # max-log: bit-exact, closed form and level metrics alike
    np.testing.assert_array_equal(oracle.llr(x, order, s2, method="maxlog"), g[key + "_closed"])
    np.testing.assert_array_equal(
        oracle.llr(x, order, s2, method="maxlog", closed_form=False), g[key + "_levels_maxlog"]
    )
    # the reference's own identity: closed form == level metrics, bit for bit
    np.testing.assert_array_equal(g[key + "_closed"], g[key + "_levels_maxlog"])
    # exact: within float32 rounding of exp/log (spec tolerance)
    np.testing.assert_allclose(oracle.llr(x, order, s2, method="exact"), g[key + "_exact"],
                               rtol=1e-5, atol=1e-6)  # fmt: skip


def test_llr_oracle_frames():
    """Per-frame noise: each frame equals the single-variance call."""
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(3 * 50) + 1j * rng.standard_normal(3 * 50)).astype(np.complex64)
    s2 = np.array([1.0, 10.0, 100.0], np.float32)
    for method in ("maxlog", "exact"):
        whole = oracle.llr(x, 16, s2, method=method, frame_len=50)
        for f in range(3):
            one = oracle.llr(x[50 * f : 50 * f + 50], 16, s2[f], method=method)
            np.testing.assert_array_equal(whole[50 * f : 50 * f + 50], one)


@pytest.mark.parametrize("name", ["A", "B", "C"])
def test_schedule_matches_reference(golden_ldpc, name):
    g = golden_ldpc
    spec = W.CODES[name]
    base = spec.base()
    np.testing.assert_array_equal(base, g[f"{name}_base"])
    checks, variables = oracle.lift(base, spec.z)
    m, n = base.shape[0] * spec.z, base.shape[1] * spec.z
    row_ptr, cols, layer_ptr = oracle.schedule(checks, variables, m, n)
    assert digest(np.concatenate([row_ptr, cols])) == g[f"{name}_schedule_digest"]
    np.testing.assert_array_equal(layer_ptr, g[f"{name}_layer_ptr"])


def _check_case(g, prefix, bits, post, valid, iters):
    np.testing.assert_array_equal(iters, g[prefix + "_iters"])
    np.testing.assert_array_equal(valid, g[prefix + "_valid"])
    np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), g[prefix + "_bits_packed"])
    np.testing.assert_array_equal(post[0], g[prefix + "_post_first"])
    assert digest(post) == g[prefix + "_post_digest"]


def _qc_llrs(g, name):
    spec = W.CODES[name]
    frames, order = int(g[f"{name}_frames"]), int(g[f"{name}_order"])
    batch = W.coded_batch(spec, frames, order, float(g[f"{name}_ebn0"]), seed=7)
    assert digest(batch.symbols) == g[f"{name}_symbols_digest"]
    method = str(g[f"{name}_llr_method"])
    llrs = np.stack([
        oracle.llr(batch.symbols[f], order, oracle.inv_s2(batch.noise_var[f]), method=method).reshape(-1)
        for f in range(frames)
    ])  # fmt: skip
    return llrs


@pytest.mark.parametrize("name", ["A", "B", "C"])
def test_decode_oracle_matches_reference(golden_ldpc, name):
    """Coded batches of codes A/B/C: LLRs (oracle demapper) and the min-sum
    decode (oracle decoder) against the reference's, bit for bit."""
    g = golden_ldpc
    llrs = _qc_llrs(g, name)
    if g[f"{name}_llrs"].size:
        if str(g[f"{name}_llr_method"]) == "exact":
            np.testing.assert_allclose(llrs, g[f"{name}_llrs"], rtol=1e-5, atol=1e-6)
            llrs = g[f"{name}_llrs"]  # decode the reference's own LLRs
        else:
            np.testing.assert_array_equal(llrs, g[f"{name}_llrs"])
    else:
        assert digest(llrs) == g[f"{name}_llrs_digest"]
    spec = W.CODES[name]
    checks, variables = oracle.lift(spec.base(), spec.z)
    m, n = spec.base().shape[0] * spec.z, spec.base().shape[1] * spec.z
    row_ptr, cols, _ = oracle.schedule(checks, variables, m, n)
    bits, post, valid, iters = oracle.decode(
        llrs, (row_ptr, cols, n), k=int(g[f"{name}_k"]),
        max_iterations=int(g[f"{name}_max_iterations"]),
    )  # fmt: skip
    _check_case(g, name, bits, post, valid, iters)


@pytest.mark.parametrize("which", ["dvbs2s", "pon"])
@pytest.mark.parametrize("early_stop", [False, True])
def test_reference_kat(golden_ldpc, which, early_stop):
    """The reference's own bit-exactness cases (DVB-S2 short 1/2, PON; seed-1
    LLRs; ``MinSum(0.75, 0.05, 12)``) through the oracle."""
    g = golden_ldpc
    m, N, n, k = (int(g[f"{which}_{s}"]) for s in ("m", "N", "n", "k"))
    llrs = kat_llrs(n)
    assert digest(llrs) == g[f"{which}_llrs_digest"]
    row_ptr, cols, layer_ptr = oracle.schedule(g[f"{which}_checks"], g[f"{which}_variables"], m, N)
    assert digest(np.concatenate([row_ptr, cols])) == g[f"{which}_schedule_digest"]
    np.testing.assert_array_equal(layer_ptr, g[f"{which}_layer_ptr"])
    bits, post, valid, iters = oracle.decode(
        llrs, (row_ptr, cols, N), k=k, scale=0.75, offset=0.05, max_iterations=12,
        early_stop=early_stop,
    )  # fmt: skip
    _check_case(g, f"{which}_es{int(early_stop)}", bits, post, valid, iters)


@pytest.mark.parametrize("which", ["dvbs2s", "pon"])
@pytest.mark.parametrize("early_stop", [False, True])
def test_nonfinite_llrs(golden_ldpc, which, early_stop):
    """LLRs holding +-inf and a NaN (``ldpc_nonfinite.npz``): the oracle
    skips NaN magnitudes in min1/min2 as the reference does; posteriors
    equal the reference's, NaN where it has NaN."""
    from tests.conftest import GOLDEN

    g, nf = golden_ldpc, np.load(GOLDEN / "ldpc_nonfinite.npz")
    m, N, k = (int(g[f"{which}_{s}"]) for s in ("m", "N", "k"))
    row_ptr, cols, _ = oracle.schedule(g[f"{which}_checks"], g[f"{which}_variables"], m, N)
    bits, post, valid, iters = oracle.decode(nf[f"nf_{which}_llrs"], (row_ptr, cols, N), k=k, max_iterations=12,
                                             early_stop=early_stop)  # fmt: skip
    p = f"nf_{which}_es{int(early_stop)}"
    np.testing.assert_array_equal(iters, nf[p + "_iters"])
    np.testing.assert_array_equal(valid, nf[p + "_valid"])
    np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), nf[p + "_bits"])
    np.testing.assert_array_equal(post, nf[p + "_post"])


def test_oracle_threads_do_not_change_results(golden_ldpc):
    g = golden_ldpc
    llrs = kat_llrs(int(g["pon_n"]))
    m, N = int(g["pon_m"]), int(g["pon_N"])
    row_ptr, cols, _ = oracle.schedule(g["pon_checks"], g["pon_variables"], m, N)
    outs = [oracle.decode(llrs, (row_ptr, cols, N), k=int(g["pon_k"]), max_iterations=5, threads=t)
            for t in (1, 3)]  # fmt: skip
    for a, b in zip(*outs, strict=True):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("tag", SP_TAGS)
@pytest.mark.parametrize("early_stop", [False, True])
def test_sum_product_oracle_matches_reference(golden_ldpc, golden_sp, tag, early_stop):
    """The oracle's sum-product rule against the reference's CPU decoder."""
    g, sp = golden_ldpc, golden_sp
    which = str(sp[f"sp_{tag}_code"])
    m, N, k = (int(g[f"{which}_{s}"]) for s in ("m", "N", "k"))
    row_ptr, cols, _ = oracle.schedule(g[f"{which}_checks"], g[f"{which}_variables"], m, N)
    bits, post, valid, iters = oracle.decode(
        sp[f"sp_{tag}_llrs"], (row_ptr, cols, N), k=k, sum_product=True,
        max_iterations=int(sp[f"sp_{tag}_max_iterations"]), early_stop=early_stop,
    )  # fmt: skip
    check_sum_product(sp, f"sp_{tag}_es{int(early_stop)}", bits, post, valid, iters,
                      saturated=tag in SP_SATURATED)  # fmt: skip


def test_dvbs2_normal_oracle_and_encoder():
    """DVB-S2 normal-frame rate 1/2, the code of the reference's LDPC
    benchmark: schedule, accumulator encoding, QPSK LLRs and MinSum() decode
    against the reference (``dvbs2_normal.npz``)."""
    from commkit_gb300.workloads import encode_accumulate
    from tests.conftest import GOLDEN
    from tests.golden.make_golden import dvbs2_symbols

    d = dict(np.load(GOLDEN / "dvbs2_normal.npz"))
    m, N, n, k = (int(d[f"dvbs2n_{s}"]) for s in ("m", "N", "n", "k"))
    row_ptr, cols, layer_ptr = oracle.schedule(d["dvbs2n_checks"], d["dvbs2n_variables"], m, N)
    np.testing.assert_array_equal(layer_ptr, d["dvbs2n_layer_ptr"])
    info = np.unpackbits(d["dvbs2n_info"], axis=1)[:, :k].astype(np.int8)
    words = encode_accumulate(d["dvbs2n_checks"], d["dvbs2n_variables"], m, k, info)
    np.testing.assert_array_equal(np.packbits(words.astype(np.uint8), axis=1), d["dvbs2n_words"])
    rx, nv = dvbs2_symbols(words[:2], 1.5, seed=5)
    llrs = oracle.llr(rx.reshape(-1), 4, oracle.inv_s2(nv)).reshape(2, -1)
    assert digest(llrs) == d["dvbs2n_llrs_digest"]
    bits, post, valid, iters = oracle.decode(llrs, (row_ptr, cols, N), k=k, max_iterations=50)
    _check_case(d, "dvbs2n", bits, post, valid, iters)


@pytest.mark.parametrize("name", ["w64qc", "w64csr", "dvbs2n910"])
def test_wide_rows_oracle_matches_reference(name):
    """Codes with rows above 27 edges (``ldpc_wide.npz``: DVB-S2 normal 9/10,
    and seeded codes with rows of 64): the oracle's schedule and its min-sum
    (bit-exact) and sum-product decodes against the reference's."""
    from tests.conftest import GOLDEN
    from tests.golden.make_golden import wide_llrs

    g = dict(np.load(GOLDEN / "ldpc_wide.npz"))
    m, N, n, k = (int(g[f"{name}_{s}"]) for s in ("m", "N", "n", "k"))
    row_ptr, cols, layer_ptr = oracle.schedule(g[f"{name}_checks"], g[f"{name}_variables"], m, N)
    np.testing.assert_array_equal(layer_ptr, g[f"{name}_layer_ptr"])
    assert digest(np.concatenate([row_ptr, cols]).astype(np.int32)) == g[f"{name}_schedule_digest"]
    assert np.diff(row_ptr).max() == int(g[f"{name}_max_degree"]) > 27
    llrs = wide_llrs(name, n)
    assert digest(llrs) == g[f"{name}_llrs_digest"]
    for tag, kw in (("ms", {}), ("ms2", dict(scale=0.75, offset=0.05, max_iterations=12, early_stop=False))):
        bits, post, valid, iters = oracle.decode(llrs, (row_ptr, cols, N), k=k, **kw)
        key = f"{name}_{tag}"
        np.testing.assert_array_equal(iters, g[key + "_iters"])
        np.testing.assert_array_equal(valid, g[key + "_valid"])
        np.testing.assert_array_equal(np.packbits(bits.astype(np.uint8), axis=1), g[key + "_bits_packed"])
        np.testing.assert_array_equal(post[0], g[key + "_post_first"])
        assert digest(post) == g[key + "_post_digest"]
    for tag, es in (("sp0", False), ("sp1", True)):
        bits, post, valid, iters = oracle.decode(llrs, (row_ptr, cols, N), k=k, sum_product=True,
                                                 max_iterations=10, early_stop=es)  # fmt: skip
        check_sum_product(g, f"{name}_{tag}", bits, post, valid, iters, saturated=True)
