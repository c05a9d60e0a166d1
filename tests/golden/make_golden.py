"""Generate the golden fixtures of ``tests/golden/`` by running the reference.

Run once, where the reference source tree is available::

    python tests/golden/make_golden.py /path/to/commkit-reference

It imports ``commkit`` from that tree with a no-op ``numba`` stand-in
(``njit`` -> identity, ``prange`` -> ``range``), so the reference's Numba
kernels run as plain Python on numpy float32 scalars, as its own CI runs
them with ``NUMBA_DISABLE_JIT=1`` (``.github/workflows/ci.yml:91-116``).
Every output here is the reference's own result on seeded inputs:

* ``qam_tables.npz``: Gray QAM points, labels and the per-axis demapper
  tables (``commkit/mapping/_lattice.py:100-124``, ``_demap.py:82-106,355``)
  for 4/16/64/256-QAM;
* ``llr_golden.npz``: LLRs of seeded symbols (plus ties at level midpoints
  and far-out points) from the closed-form max-log kernel and the
  level-metric max-log and exact kernels (``commkit/mapping/_numba_llr.py``);
* ``ldpc_golden.npz``: the first-fit schedules and min-sum decodes of the
  seeded codes A, B and C (``commkit_gb300.workloads``) and of the
  reference's own known-answer cases, DVB-S2 short 1/2 and PON with
  ``MinSum(0.75, 0.05, 12)`` on ``1.8 + 1.5 N(0,1)`` LLRs of seed 1
  (``tests/coding/test_ldpc_kernel.py:16-34``);
* ``ldpc_sp_golden.npz``: sum-product decodes (five iterations, with and
  without early stop) of DVB-S2 short 1/2 on the reference's own
  GPU-vs-CPU input (``0.8 + 1.5 N(0,1)``, seed 2, four frames;
  ``tests/coding/test_ldpc_kernel.py:37-45``) and of PON on two frames of
  the same distribution (``--only=sp`` writes just this file);
* ``llr_mpoint_golden.npz``: points, labels and priors of PSK, 8-QAM,
  cross QAM, PAM, Maxwell-Boltzmann-shaped QAM and a random labelled
  constellation with a prior, and their LLRs through the reference's
  ``Constellation.llr`` on CPU input (``--only=mpoint``);
* ``dvbs2_normal.npz``: the DVB-S2 normal-frame rate-1/2 code of the
  reference's LDPC benchmark, reference encodings of seeded words and the
  reference's ``MinSum()`` decode of two QPSK frames at Es/N0 1.5 dB
  (``--only=dvbs2``);
* ``gmi_golden.npz``: the reference's ``gmi`` / ``ngmi`` of seeded 16-QAM,
  8-PSK and shaped 64-QAM LLRs (``--only=gmi``);
* ``api_signatures.json``: parameter names, kinds and defaults of the
  reference's public calls on this path (``--only=api``);
* ``ldpc_nonfinite.npz``: min-sum on LLRs with infinities and a NaN,
  DVB-S2 short 1/2 and PON (``--only=nonfinite``);
* ``ldpc_wide.npz``: codes with rows above 27 edges (DVB-S2 normal 9/10,
  rows of 30; two seeded codes with rows of 64, circulant and not): the
  reference's schedules and its min-sum and sum-product decodes
  (``--only=wide``);
* ``registry_calls.npz``: the reference's own launcher calls, recorded at
  its kernel registry while its ``compute_llr`` and ``decode`` run their GPU
  route on stand-in CuPy arrays (the tables, ``inv_s2`` from ``esn0_db``,
  schedules and padded posteriors its host code builds), with its CPU
  results on the same inputs (``--only=registry``);
* ``ldpc_generator.npz``: three codes whose parity part is not invertible
  (a cycle-free code, a random code with a redundant check, a circulant
  code whose block columns have weight two), with the reference's ``k``,
  information and pivot columns, encodings of seeded words and min-sum
  decodes (``--only=generator``).

Large outputs are stored as SHA-256 digests of their bytes (negative zeros
folded to +0) plus their first frame; inputs drawn from ``default_rng``
are stored as a digest and regenerated by the tests.
"""

from __future__ import annotations

import hashlib
import sys
import time
import types
from concurrent.futures import ProcessPoolExecutor
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]


def digest(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    if a.dtype.kind == "f":
        a = np.where(a == 0, np.zeros_like(a), a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def _numba_stand_in() -> None:
    if "numba" in sys.modules:
        return
    mod = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    class _Any:
        def __getattr__(self, name):
            return self

        def __call__(self, *a, **k):
            return self

        def __getitem__(self, k):
            return self

    mod.njit = mod.jit = njit
    mod.vectorize = mod.guvectorize = lambda *a, **k: (lambda f: f)
    mod.prange = range
    mod.get_num_threads = lambda: 1
    mod.set_num_threads = lambda n: None
    mod.types = mod.config = _Any()
    sys.modules["numba"] = mod


def _import_reference(ref: str):
    _numba_stand_in()
    if ref not in sys.path:
        sys.path.insert(0, ref)
    if str(REPO) not in sys.path:
        sys.path.insert(0, str(REPO))
    import commkit

    return commkit


# ---------------------------------------------------------------------------


def qam_tables(ref: str) -> dict:
    _import_reference(ref)
    from commkit.mapping import Constellation
    from commkit.mapping._demap import _opposite_levels, _packed_labels

    out = {}
    for order in (4, 16, 64, 256):
        c = Constellation.qam(order)
        out[f"q{order}_points"] = np.asarray(c.points)
        out[f"q{order}_bit_labels"] = np.asarray(c.bit_labels, np.int8)
        out[f"q{order}_power"] = np.float64(c.power())
        for name, ax in zip(("re", "im"), c._axes, strict=True):
            lo, hi = _opposite_levels(ax.labels)
            out[f"q{order}_{name}_levels"] = ax.levels.astype(np.float32)
            out[f"q{order}_{name}_labels"] = _packed_labels(ax.labels).astype(np.int32)
            out[f"q{order}_{name}_lo"] = lo
            out[f"q{order}_{name}_hi"] = hi
            out[f"q{order}_{name}_pos"] = ax.bits.astype(np.int32)
    return out


def llr_symbols(order: int, seed: int, n: int = 480) -> np.ndarray:
    """Seeded symbols: noisy points, exact midpoints between levels, far-out
    points and zeros."""
    from commkit_gb300.workloads import gray_qam_points

    rng = np.random.default_rng(seed)
    pts = gray_qam_points(order).astype(np.complex64)
    x = pts[rng.integers(0, order, n)] + (0.15 * rng.standard_normal(n)
                                          + 0.15j * rng.standard_normal(n)).astype(np.complex64)  # fmt: skip
    lev = np.unique(pts.real)
    mids = ((lev[1:] + lev[:-1]) / 2).astype(np.float32)
    special = [complex(a, b) for a in mids for b in mids[:2]]
    special += [complex(3.0 * lev[-1], -4.0 * lev[-1]), complex(-50.0, 50.0), 0j, complex(lev[0], lev[-1])]
    return np.concatenate([x.astype(np.complex64), np.asarray(special, np.complex64)])


def llr_golden(ref: str) -> dict:
    _import_reference(ref)
    from commkit.mapping import Constellation
    from commkit.mapping import _numba_llr as K
    from commkit.mapping._demap import _half_indices, _log_prior, _opposite_levels, _packed_labels

    out = {}
    for order in (4, 16, 64, 256):
        c = Constellation.qam(order)
        re, im = c._axes
        k = re.bits.size + im.bits.size
        for ni, nv in enumerate((0.5, 0.05, 1e-3)):
            x = llr_symbols(order, seed=100 + 10 * order + ni)
            inv_s2 = np.float32(1.0 / max(nv, 1e-20))
            xr, xi = x.real, x.imag
            closed = np.empty((x.size, k), np.float32)
            args = []
            for a in (re, im):
                lo, hi = _opposite_levels(a.labels)
                args += [a.levels.astype(np.float32), _packed_labels(a.labels), lo, hi,
                         a.bits.astype(np.int64)]  # fmt: skip
            K.llr_separable_maxlog_kernel(xr, xi, *args, inv_s2, closed)
            tabs = (re.levels.astype(np.float32), im.levels.astype(np.float32),
                    _log_prior(re.pmf, re.levels.size), _log_prior(im.pmf, im.levels.size),
                    _half_indices(re.labels), _half_indices(im.labels),
                    re.bits.astype(np.int64), im.bits.astype(np.int64))  # fmt: skip
            levels_max = np.empty((x.size, k), np.float32)
            K.llr_separable_kernel(xr, xi, *tabs, inv_s2, False, levels_max)
            exact = np.empty((x.size, k), np.float32)
            K.llr_separable_kernel(xr, xi, *tabs, inv_s2, True, exact)
            key = f"q{order}_n{ni}"
            out[key + "_x"] = x
            out[key + "_nv"] = np.float64(nv)
            out[key + "_inv_s2"] = inv_s2
            out[key + "_closed"] = closed
            out[key + "_levels_maxlog"] = levels_max
            out[key + "_exact"] = exact
    return out


def dvbs2_symbols(words: np.ndarray, esn0_db: float, seed: int) -> tuple[np.ndarray, float]:
    """Gray QPSK of codewords through complex AWGN at ``esn0_db``:
    ``(symbols complex64, noise_var)``, seeded (``numpy.random.default_rng``)."""
    from commkit_gb300.workloads import awgn, map_bits

    nv = 10.0 ** (-esn0_db / 10.0)
    return awgn(map_bits(words, 4), nv, np.random.default_rng(seed)), nv


def dvbs2_case(ref: str) -> dict:
    """DVB-S2 normal-frame rate 1/2 (n = 64800, k = 32400), the code of the
    reference's LDPC benchmark (``benchmarks/bench_coding.py:37-38,55-56``):
    its parity-check edges, three reference encodings of seeded words, and
    the reference's ``MinSum()`` decode of two of them over QPSK at Es/N0
    1.5 dB (its benchmark's operating point)."""
    _import_reference(ref)
    from commkit.coding import LDPCCode, MinSum, decode, encode
    from commkit.mapping import Constellation, compute_llr

    code = LDPCCode.dvbs2("1/2")
    rng = np.random.default_rng(4)
    info = rng.integers(0, 2, size=(3, code.k), dtype=np.int8)
    words = np.asarray(encode(info.reshape(-1), code=code), np.int8).reshape(3, -1)
    rx, nv = dvbs2_symbols(words[:2], 1.5, seed=5)
    llrs = np.asarray(compute_llr(rx, noise_var=nv, constellation=Constellation.qam(4)), np.float32)
    llrs = llrs.reshape(2, -1)
    res = decode(llrs.reshape(-1), code=code, method=MinSum())
    post = np.asarray(res.llrs, np.float32).reshape(2, -1)
    row_ptr, cols, layer_ptr = code._schedule
    return {
        "dvbs2n_checks": code.checks.astype(np.int32), "dvbs2n_variables": code.variables.astype(np.int32),
        "dvbs2n_m": np.int64(code.num_checks), "dvbs2n_N": np.int64(code.num_variables),
        "dvbs2n_n": np.int64(code.n), "dvbs2n_k": np.int64(code.k),
        "dvbs2n_layer_ptr": layer_ptr.astype(np.int32),
        "dvbs2n_info": np.packbits(info.astype(np.uint8), axis=1),
        "dvbs2n_words": np.packbits(words.astype(np.uint8), axis=1),
        "dvbs2n_llrs_digest": digest(llrs), "dvbs2n_post_digest": digest(post), "dvbs2n_post_first": post[0],
        "dvbs2n_bits_packed": np.packbits(np.asarray(res.bits, np.uint8).reshape(2, -1), axis=1),
        "dvbs2n_valid": np.asarray(res.valid, bool).reshape(-1),
        "dvbs2n_iters": np.asarray(res.iterations, np.int32).reshape(-1),
    }  # fmt: skip


def gmi_case(ref: str) -> dict:
    """The reference's ``gmi`` and ``ngmi`` (``commkit/metrics/information.py``)
    of seeded 16-QAM, 8-PSK and shaped 64-QAM LLRs, 1-D and 2-D, with a
    skipped leading symbol."""
    _import_reference(ref)
    from commkit.mapping import Constellation, compute_llr
    from commkit.metrics import gmi, ngmi

    out = {}
    cases = (("q16", Constellation.qam(16), 0.08), ("p8", Constellation.psk(8), 0.05),
             ("q64s", Constellation.qam(64).shaped(entropy=5.0), 0.02))  # fmt: skip
    for i, (name, c, nv) in enumerate(cases):
        rng = np.random.default_rng(40 + i)
        k = c.bits_per_symbol
        bits = rng.integers(0, 2, size=(2, 600 * k), dtype=np.int8)
        labels = (bits.reshape(2, 600, k).astype(np.int64) << np.arange(k - 1, -1, -1)).sum(-1)
        from commkit.mapping._demap import _packed_labels

        by_label = np.empty(c.order, complex)
        by_label[_packed_labels(c.bit_labels)] = c.points
        x = by_label[labels] + np.sqrt(nv / 2) * (rng.standard_normal((2, 600)) + 1j * rng.standard_normal((2, 600)))
        x = x.astype(np.complex64)
        llr = np.asarray(compute_llr(x, noise_var=nv, constellation=c), np.float32)
        out[f"{name}_llrs"], out[f"{name}_bits"] = llr, bits
        out[f"{name}_gmi2"] = np.asarray(gmi(llr, bits, constellation=c), np.float64)
        out[f"{name}_ngmi2"] = np.asarray(ngmi(llr, bits, constellation=c), np.float64)
        out[f"{name}_gmi1"] = np.float64(gmi(llr[0], bits[0], constellation=c))
        out[f"{name}_gmi1_skip"] = np.float64(gmi(llr[0], bits[0], constellation=c, num_skip_symbols=5))
    return out


# Constellations of the M-point and prior-weighted demapping paths:
# (name, builder over the reference's Constellation).
CONSTELLATIONS = (
    ("psk2", lambda C: C.psk(2)),
    ("psk8", lambda C: C.psk(8)),
    ("psk16", lambda C: C.psk(16)),
    ("qam2", lambda C: C.qam(2)),
    ("qam8", lambda C: C.qam(8)),
    ("qam32", lambda C: C.qam(32)),
    ("qam128", lambda C: C.qam(128)),
    ("qam512", lambda C: C.qam(512)),
    ("pam4", lambda C: C.pam(4)),
    ("pam8u", lambda C: C.pam(8, unipolar=True)),
    ("qam16nu", lambda C: C.qam(16).shaped(nu=0.05)),
    ("qam64h5", lambda C: C.qam(64).shaped(entropy=5.0)),
    ("qam32h4", lambda C: C.qam(32).shaped(entropy=4.5)),
    ("custom16", None),
)


def _custom16(C):
    """16 random points, a random labelling and a random prior."""
    rng = np.random.default_rng(99)
    pts = rng.standard_normal(16) + 1j * rng.standard_normal(16)
    perm = rng.permutation(16)
    labels = ((perm[:, None] >> np.arange(3, -1, -1)) & 1).astype(np.int8)
    pmf = rng.uniform(0.2, 1.0, 16)
    return C(pts, bit_labels=labels, pmf=pmf / pmf.sum())


def mpoint_golden(ref: str) -> dict:
    """Tables and CPU LLRs of the constellations above through the
    reference's own ``Constellation.llr`` (its CPU routing: per-axis kernels
    for separable lattices, ``llr_kernel`` over every point otherwise), on
    seeded noisy symbols plus the origin and far-out points, max-log and
    exact, at two noise levels."""
    _import_reference(ref)
    from commkit.mapping import Constellation

    out = {}
    for ci, (name, build) in enumerate(CONSTELLATIONS):
        c = _custom16(Constellation) if build is None else build(Constellation)
        out[f"{name}_points"] = np.asarray(c.points)
        out[f"{name}_bit_labels"] = np.asarray(c.bit_labels, np.int8)
        out[f"{name}_pmf"] = np.zeros(0) if c.pmf is None else np.asarray(c.pmf, np.float64)
        out[f"{name}_power"] = np.float64(c.power())
        out[f"{name}_entropy"] = np.float64(c.entropy)
        out[f"{name}_separable"] = np.bool_(c._axes is not None)
        rng = np.random.default_rng(1000 + ci)
        n = 300
        pts = np.asarray(c.points)
        idx = rng.integers(0, c.order, n)
        if c.is_complex:
            x = pts[idx] + 0.2 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
            x = np.concatenate([x, [0j, 40 - 30j, -0.5 + 7j]]).astype(np.complex64)
        else:
            x = pts[idx] + 0.2 * rng.standard_normal(n)
            x = np.concatenate([x, [0.0, 40.0, -9.0]]).astype(np.float32)
        out[f"{name}_x"] = x
        for ni, nv in enumerate((0.3, 0.02)):
            for method in ("maxlog", "exact"):
                llr = np.asarray(c.llr(x, noise_var=nv, method=method), np.float32)
                out[f"{name}_n{ni}_{method}"] = llr.reshape(x.size, -1)
            out[f"{name}_n{ni}_nv"] = np.float64(nv)
    return out


def _decode_case(ref: str, code, llrs: np.ndarray, method) -> dict:
    from commkit.coding import decode

    res = decode(llrs.reshape(-1), code=code, method=method)
    B = llrs.shape[0]
    post = np.asarray(res.llrs, np.float32).reshape(B, -1)
    return {
        "post_digest": digest(post),
        "post_first": post[0].copy(),
        "bits_packed": np.packbits(np.asarray(res.bits, np.uint8).reshape(B, -1), axis=1),
        "valid": np.asarray(res.valid, bool),
        "iters": np.asarray(res.iterations, np.int32),
    }


def ldpc_qc_case(ref: str, name: str, frames: int, order: int, ebn0: float,
                 max_iterations: int, method_name: str) -> dict:  # fmt: skip
    """A seeded code of ``commkit_gb300.workloads`` through the reference:
    schedule, encode (checked against the workload encoder), LLRs, decode."""
    commkit = _import_reference(ref)
    from commkit.coding import LDPCCode, MinSum, encode
    from commkit.coding import ldpc as ldpc_module
    from commkit.mapping import Constellation, compute_llr

    from commkit_gb300 import workloads as W

    spec = W.CODES[name]
    base = spec.base()
    ldpc_module._MAX_INVERSE = max(ldpc_module._MAX_INVERSE, base.shape[0] * spec.z)
    code = LDPCCode.quasi_cyclic(base, lifting=spec.z)
    row_ptr, cols, layer_ptr = code._schedule
    batch = W.coded_batch(spec, frames, order, ebn0, seed=7)
    ref_words = np.asarray(encode(batch.info.reshape(-1), code=code)).reshape(frames, -1)
    ours = W.encode_qc(base, spec.z, batch.info)
    assert np.array_equal(ref_words, ours), "workload encoder differs from the reference's"
    c = Constellation.qam(order)
    method = "exact" if method_name == "exact" else "maxlog"
    llrs = np.stack([
        np.asarray(compute_llr(batch.symbols[f], noise_var=float(batch.noise_var[f]),
                               constellation=c, method=method), np.float32)
        for f in range(frames)
    ])  # fmt: skip
    case = _decode_case(ref, code, llrs, MinSum(max_iterations=max_iterations))
    out = {f"{name}_{k}": v for k, v in case.items()}
    out.update({
        f"{name}_base": base, f"{name}_z": np.int64(spec.z), f"{name}_order": np.int64(order),
        f"{name}_ebn0": np.float64(ebn0), f"{name}_frames": np.int64(frames),
        f"{name}_max_iterations": np.int64(max_iterations), f"{name}_llr_method": method,
        f"{name}_layer_ptr": layer_ptr.astype(np.int32),
        f"{name}_schedule_digest": digest(np.concatenate([row_ptr, cols]).astype(np.int32)),
        f"{name}_symbols_digest": digest(batch.symbols),
        f"{name}_llrs": llrs if llrs.size <= 40000 else np.zeros(0, np.float32),
        f"{name}_llrs_digest": digest(llrs), f"{name}_k": np.int64(code.k),
    })  # fmt: skip
    del commkit
    return out


def kat_case(ref: str, which: str) -> dict:
    """The reference's bit-exactness cases (``tests/coding/test_ldpc_kernel.py:16-34``)."""
    _import_reference(ref)
    from commkit.coding import LDPCCode, MinSum

    code = LDPCCode.dvbs2("1/2", frame="short") if which == "dvbs2s" else LDPCCode.pon()
    rng = np.random.default_rng(1)
    llrs = (1.8 + 1.5 * rng.standard_normal((6, code.n))).astype(np.float32)
    row_ptr, cols, layer_ptr = code._schedule
    out = {
        f"{which}_checks": code.checks.astype(np.int32),
        f"{which}_variables": code.variables.astype(np.int32),
        f"{which}_m": np.int64(code.num_checks), f"{which}_N": np.int64(code.num_variables),
        f"{which}_n": np.int64(code.n), f"{which}_k": np.int64(code.k),
        f"{which}_layer_ptr": layer_ptr.astype(np.int32),
        f"{which}_schedule_digest": digest(np.concatenate([row_ptr, cols]).astype(np.int32)),
        f"{which}_llrs_digest": digest(llrs),
    }  # fmt: skip
    for es in (False, True):
        case = _decode_case(ref, code, llrs,
                            MinSum(scale=0.75, offset=0.05, max_iterations=12, early_stop=es))  # fmt: skip
        out.update({f"{which}_es{int(es)}_{k}": v for k, v in case.items()})
    return out


def sp_case(ref: str, which: str, tag: str, mean: float, seed: int, frames: int,
            iterations: int) -> dict:  # fmt: skip
    """Sum-product through the reference's CPU decoder on ``frames`` frames of
    ``mean + 1.5 N(0,1)`` LLRs (``default_rng(seed)``), ``iterations`` at
    most, with and without early stop."""
    _import_reference(ref)
    from commkit.coding import LDPCCode, SumProduct, decode

    code = LDPCCode.dvbs2("1/2", frame="short") if which == "dvbs2s" else LDPCCode.pon()
    rng = np.random.default_rng(seed)
    llrs = (mean + 1.5 * rng.standard_normal((frames, code.n))).astype(np.float32)
    out = {f"sp_{tag}_code": which, f"sp_{tag}_llrs": llrs, f"sp_{tag}_max_iterations": np.int64(iterations)}
    for es in (False, True):
        method = SumProduct(max_iterations=iterations, early_stop=es)
        case = _decode_case(ref, code, llrs, method)
        case.pop("post_first")
        out.update({f"sp_{tag}_es{int(es)}_{k}": v for k, v in case.items()})
        res = decode(llrs.reshape(-1), code=code, method=method)
        out[f"sp_{tag}_es{int(es)}_post"] = np.asarray(res.llrs, np.float32).reshape(frames, -1)
    return out


def nonfinite_case(ref: str, which: str) -> dict:
    """Min-sum through the reference on LLRs holding infinities and a NaN:
    3 frames of ``m + 1.5 N(0,1)`` (``default_rng(5)``, the all-zero word; m
    = 1.8 for DVB-S2, 3.0 for PON)
    with 1 % of the entries set to +inf (frame 0: it still converges), to
    +-inf (frame 1) or to +inf plus one NaN (frame 2); 12 iterations at
    most, with and without early stop.  A NaN Q (from the NaN input, or
    inf - inf inside the decoder) is skipped by the reference's min1/min2
    comparisons."""
    _import_reference(ref)
    from commkit.coding import LDPCCode, MinSum, decode

    code = LDPCCode.dvbs2("1/2", frame="short") if which == "dvbs2s" else LDPCCode.pon()
    rng = np.random.default_rng(5)
    mean = 1.8 if which == "dvbs2s" else 3.0
    llrs = (mean + 1.5 * rng.standard_normal((3, code.n))).astype(np.float32)
    hit = rng.random(llrs.shape) < 0.01
    sign = np.where(rng.random(llrs.shape) < 0.5, -1.0, 1.0)
    sign[[0, 2]] = 1.0
    llrs[hit] = (sign * np.inf)[hit].astype(np.float32)
    llrs[2, code.n - 5] = np.nan  # a parity variable: late in its rows, after min1 is set
    out = {f"nf_{which}_llrs": llrs}
    for es in (False, True):
        method = MinSum(max_iterations=12, early_stop=es)
        res = decode(llrs.reshape(-1), code=code, method=method)
        out[f"nf_{which}_es{int(es)}_post"] = np.asarray(res.llrs, np.float32).reshape(3, -1)
        out[f"nf_{which}_es{int(es)}_bits"] = np.packbits(np.asarray(res.bits, np.uint8).reshape(3, -1), axis=1)
        out[f"nf_{which}_es{int(es)}_valid"] = np.asarray(res.valid, bool)
        out[f"nf_{which}_es{int(es)}_iters"] = np.asarray(res.iterations, np.int32)
    return out


# (tag, code, mean, seed, frames, iterations): the reference's own GPU-vs-CPU
# case (tests/coding/test_ldpc_kernel.py:37-45), the circulant path (PON),
# and both codes at an SNR where some frames stop early.
SP_CASES = (
    ("dvbs2s", "dvbs2s", 0.8, 2, 4, 5),
    ("pon", "pon", 0.8, 2, 2, 5),
    ("dvbs2s_hi", "dvbs2s", 1.8, 1, 4, 10),
    ("pon_hi", "pon", 3.0, 1, 2, 10),
)


API_CALLABLES = (
    ("mapping", "compute_llr"), ("coding", "decode"), ("coding", "encode"), ("metrics", "gmi"),
    ("metrics", "ngmi"), ("coding", "error_rate_curve"), ("mapping", "Constellation.llr"),
    ("mapping", "Constellation.qam"), ("mapping", "Constellation.psk"), ("mapping", "Constellation.pam"),
    ("mapping", "Constellation.shaped"), ("mapping", "Constellation"), ("coding", "LDPCCode"),
    ("coding", "LDPCCode.quasi_cyclic"), ("coding", "MinSum"), ("coding", "SumProduct"),
)  # fmt: skip


def api_signatures(ref: str) -> dict:
    """Parameter names, kinds and defaults of the reference's public calls on
    this path (the drop-in surface), for the signature test."""
    import importlib
    import inspect

    _import_reference(ref)
    out = {}
    for mod, name in API_CALLABLES:
        obj = importlib.import_module(f"commkit.{mod}")
        for part in name.split("."):
            obj = getattr(obj, part)
        params = []
        for pname, prm in inspect.signature(obj).parameters.items():
            if pname == "self":
                continue
            default = None if prm.default is inspect.Parameter.empty else repr(prm.default)
            params.append([pname, prm.kind.name, default])
        out[f"{mod}.{name}"] = params
    return out


def generator_codes() -> dict:
    """``name -> (checks, variables, m, N)`` of the three seeded codes of
    ``ldpc_generator.npz``, each with a parity part that is not invertible."""
    out = {}
    tree = [[0, 1, 3], [3, 4, 5], [1, 2, 6], [5, 7, 8]]
    r = np.concatenate([[i] * len(row) for i, row in enumerate(tree)])
    out["tree"] = (r, np.concatenate(tree), 4, 9)
    # 23 random checks on 48 bits (column weight 2 or 3), then their first
    # two rows' sum as a 24th check: rank 23 at most.
    rng = np.random.default_rng(21)
    m, n = 23, 48
    h = np.zeros((m + 1, n), np.int8)
    for c in range(n):
        h[rng.choice(m, size=int(rng.integers(2, 4)), replace=False), c] = 1
    for i in range(m):
        while h[i].sum() < 2:
            h[i, rng.integers(n)] = 1
    h[m] = h[0] ^ h[1]
    assert h[m].sum() >= 2
    rr, cc = np.nonzero(h)
    out["redundant"] = (rr, cc, m + 1, n)
    # Circulant code, 4 x 8 base, Z = 8: every block column has two shifted
    # identities, so the block rows sum to zero and H has rank < m.
    rng = np.random.default_rng(22)
    base = -np.ones((4, 8), np.int64)
    while (base >= 0).sum(1).min() < 2:  # every check needs two bits
        base[:] = -1
        for j in range(8):
            base[rng.choice(4, size=2, replace=False), j] = rng.integers(0, 8, size=2)
    z = 8
    bi, bj = np.nonzero(base >= 0)
    lift = np.arange(z)
    rr = (bi[:, None] * z + lift).ravel()
    cc = (bj[:, None] * z + (lift + base[bi, bj][:, None]) % z).ravel()
    out["qc_even"] = (rr, cc, 4 * z, 8 * z)
    return out


def generator_case(ref: str) -> dict:
    """The reference on :func:`generator_codes`: ``k``, the information and
    pivot columns of its "dense" encoder (``commkit/coding/ldpc.py:476-481``),
    ``encode`` of 5 seeded words (``default_rng(31)``) and ``MinSum()``
    decodes of 4 frames of ``2 + 1.5 N(0,1)`` (``default_rng(32)``, the
    all-zero word)."""
    _import_reference(ref)
    from commkit.coding import LDPCCode, MinSum, decode, encode

    out = {}
    for name, (rows, cols, m, n) in generator_codes().items():
        code = LDPCCode(np.asarray(rows, np.int64), np.asarray(cols, np.int64), m, n)
        enc = code._encoder
        out[f"{name}_checks"] = np.asarray(rows, np.int32)
        out[f"{name}_variables"] = np.asarray(cols, np.int32)
        out[f"{name}_m"] = np.int32(m)
        out[f"{name}_N"] = np.int32(n)
        out[f"{name}_kind"] = np.array(enc.kind)
        out[f"{name}_k"] = np.int32(code.k)
        out[f"{name}_info"] = np.asarray(enc.info, np.int32)
        out[f"{name}_pivots"] = np.asarray(enc.parity, np.int32)
        u = np.random.default_rng(31).integers(0, 2, size=(5, code.k)).astype(np.int8)
        out[f"{name}_u"] = u
        out[f"{name}_words"] = np.asarray(encode(u.reshape(-1), code=code), np.int8).reshape(5, code.n)
        llrs = (2.0 + 1.5 * np.random.default_rng(32).standard_normal((4, code.n))).astype(np.float32)
        out[f"{name}_llrs"] = llrs
        res = decode(llrs.reshape(-1), code=code, method=MinSum())
        out[f"{name}_post"] = np.asarray(res.llrs, np.float32).reshape(4, -1)
        out[f"{name}_bits"] = np.asarray(res.bits, np.int8).reshape(4, -1)
        out[f"{name}_valid"] = np.asarray(res.valid, bool)
        out[f"{name}_iters"] = np.asarray(res.iterations, np.int32)
    return out


def wide_codes() -> dict:
    """``name -> (checks, variables, m, N)`` of two seeded codes with rows of
    64 edges, beyond the packed min-sum record's 27: a circulant code (4 x 66
    base matrix, Z = 32, the 62 information block columns all present with
    shifts of ``default_rng(41)``, a dual-diagonal parity part of identities)
    and a code without circulant structure (64 checks on 1024 bits, each
    check on 38 to 62 random information bits of ``default_rng(42)`` plus a
    dual-diagonal parity part)."""
    out = {}
    rng = np.random.default_rng(41)
    mb, nb, z = 4, 66, 32
    base = -np.ones((mb, nb), np.int64)
    base[:, : nb - mb] = rng.integers(0, z, size=(mb, nb - mb))
    for i in range(mb):
        base[i, nb - mb + i] = 0
        if i > 0:
            base[i, nb - mb + i - 1] = 0
    bi, bj = np.nonzero(base >= 0)
    lift = np.arange(z)
    rr = (bi[:, None] * z + lift).ravel()
    cc = (bj[:, None] * z + (lift + base[bi, bj][:, None]) % z).ravel()
    out["w64qc"] = (rr, cc, mb * z, nb * z)
    rng = np.random.default_rng(42)
    m, n = 64, 1024
    rows, cols = [], []
    for i in range(m):
        info = np.sort(rng.choice(n - m, size=int(rng.integers(38, 63)), replace=False))
        par = [n - m + i] if i == 0 else [n - m + i - 1, n - m + i]
        c = np.concatenate([info, par])
        rows.append(np.full(c.size, i))
        cols.append(c)
    out["w64csr"] = (np.concatenate(rows), np.concatenate(cols), m, n)
    return out


# LLR means of the wide-row cases (the all-zero word, consistent Gaussian
# LLRs: standard deviation sqrt(2 mean)), chosen so that some frames
# converge in a few iterations and others run to the limit.
WIDE_MEANS = {"w64qc": (8.0, 10.0, 10.0, 12.0), "w64csr": (9.0, 10.0, 10.0, 11.0), "dvbs2n910": (8.0, 8.5, 9.0)}


def wide_llrs(name: str, n: int) -> np.ndarray:
    """The seeded input LLRs of a wide-row case (``default_rng(43)``)."""
    means = np.asarray(WIDE_MEANS[name], np.float64)[:, None]
    rng = np.random.default_rng(43)
    return (means + np.sqrt(2.0 * means) * rng.standard_normal((means.shape[0], n))).astype(np.float32)


def wide_case(ref: str, name: str) -> dict:
    """The reference on a code with rows above 27 edges: DVB-S2 normal 9/10
    (``LDPCCode.dvbs2("9/10")``, rows of 30 edges) or one of
    :func:`wide_codes`.  Its schedule, and its ``MinSum()``,
    ``MinSum(0.75, 0.05, 12, early_stop=False)`` and ``SumProduct`` (10
    iterations, with and without early stop) decodes of :func:`wide_llrs`."""
    _import_reference(ref)
    from commkit.coding import LDPCCode, MinSum, SumProduct, decode

    if name == "dvbs2n910":
        code = LDPCCode.dvbs2("9/10")
    else:
        rows, cols, m, n = wide_codes()[name]
        code = LDPCCode(np.asarray(rows, np.int64), np.asarray(cols, np.int64), m, n)
    row_ptr, cols_s, layer_ptr = code._schedule
    llrs = wide_llrs(name, code.n)
    out = {
        f"{name}_checks": code.checks.astype(np.int32), f"{name}_variables": code.variables.astype(np.int32),
        f"{name}_m": np.int64(code.num_checks), f"{name}_N": np.int64(code.num_variables),
        f"{name}_n": np.int64(code.n), f"{name}_k": np.int64(code.k),
        f"{name}_max_degree": np.int64(np.diff(row_ptr).max()),
        f"{name}_layer_ptr": layer_ptr.astype(np.int32),
        f"{name}_schedule_digest": digest(np.concatenate([row_ptr, cols_s]).astype(np.int32)),
        f"{name}_llrs_digest": digest(llrs),
    }  # fmt: skip
    methods = {
        "ms": MinSum(),
        "ms2": MinSum(scale=0.75, offset=0.05, max_iterations=12, early_stop=False),
        "sp0": SumProduct(max_iterations=10, early_stop=False),
        "sp1": SumProduct(max_iterations=10, early_stop=True),
    }
    for tag, method in methods.items():
        case = _decode_case(ref, code, llrs, method)
        out.update({f"{name}_{tag}_{k}": v for k, v in case.items()})
        if tag.startswith("sp") or llrs.size <= 8192:
            res = decode(llrs.reshape(-1), code=code, method=method)
            out[f"{name}_{tag}_post"] = np.asarray(res.llrs, np.float32).reshape(llrs.shape[0], -1)
    return out


def _cupy_stand_in():
    """A NumPy-backed stand-in for CuPy, used only to record launcher calls:
    its arrays are a NumPy subclass whose type lives in a module named
    ``cupy``, which is how the reference's ``dispatch`` recognises device data
    (``commkit/backend.py:75-81``), so the reference's host code takes its GPU
    route and builds its launcher arguments (``commkit/mapping/_demap.py:
    184-220, 298-352``, ``commkit/coding/ldpc.py:539-588``) on the host."""
    if "cupy" in sys.modules:
        return sys.modules["cupy"]
    cp = types.ModuleType("cupy")

    class ndarray(np.ndarray):
        pass

    ndarray.__module__ = "cupy"

    def view(a):
        return np.asarray(a).view(ndarray)

    cp.ndarray = ndarray
    for name in ("float32", "float64", "complex64", "complex128", "int8", "uint8", "int32", "int64", "bool_",
                 "dtype", "newaxis", "inf", "nan", "pi"):  # fmt: skip
        setattr(cp, name, getattr(np, name))
    for name in ("asarray", "empty", "zeros", "ones", "arange", "full", "concatenate", "stack", "where",
                 "empty_like", "zeros_like", "ascontiguousarray", "abs", "log2", "sqrt", "exp", "log"):  # fmt: skip
        setattr(cp, name, (lambda f: lambda *a, **k: view(f(*a, **k)))(getattr(np, name)))
    cp.cuda = types.SimpleNamespace(Device=lambda *a: types.SimpleNamespace(id=0))
    cp.view = view
    sys.modules["cupy"] = cp
    cupyx = types.ModuleType("cupyx")
    sp = types.ModuleType("cupyx.scipy")
    cupyx.scipy = sp
    sys.modules["cupyx"] = cupyx
    sys.modules["cupyx.scipy"] = sp
    for sub in ("ndimage", "signal", "special"):
        m = types.ModuleType(f"cupyx.scipy.{sub}")
        setattr(sp, sub, m)
        sys.modules[f"cupyx.scipy.{sub}"] = m
    return cp


def _recording_registry(cuda_module, calls: list):
    """Replaces the four launcher factories of the reference's real registry
    (``commkit._cuda._KERNEL_FACTORIES``) by recorders: each call's name,
    specialisation, positional arrays (host copies; tuples kept as tuples)
    and keyword arguments go to ``calls``, and the launcher returns zeros of
    its output shape.  Returns the previous factories."""
    cp = sys.modules["cupy"]

    def host(a):
        if isinstance(a, tuple):
            return tuple(host(t) for t in a)
        return np.array(a) if isinstance(a, np.ndarray) else a

    def factory_for(name):
        def factory(**spec):
            def launch(*args, **kwargs):
                calls.append((name, dict(spec), [host(a) for a in args], dict(kwargs)))
                if name == "ldpc_layered":
                    B = args[0].shape[0]
                    return cp.zeros(B, dtype=np.int32), cp.zeros(B, dtype=np.bool_)
                n = args[0].shape[0]
                k = kwargs["k"] if name == "llr" else args[1][-1].size + args[2][-1].size
                return cp.zeros((n, k), dtype=np.float32)

            return launch

        return factory

    saved = {}
    for name in ("llr", "llr_separable_maxlog", "llr_separable", "ldpc_layered"):
        saved[name] = cuda_module._KERNEL_FACTORIES[name]
        cuda_module._KERNEL_FACTORIES[name] = factory_for(name)
    return saved


# (tag, constellation, method, Es/N0 dB, symbols): demapper calls recorded
# from the reference's GPU route; Es/N0 goes in as esn0_db, so the recorded
# inv_s2 also pins the reference's noise-variance rule (_demap.py:48-68,312).
REGISTRY_LLR_CASES = (
    ("qam16_maxlog", ("qam", 16), "maxlog", 12.0, 2048),
    ("qam64_maxlog", ("qam", 64), "maxlog", 17.5, 2048),
    ("qam16_exact", ("qam", 16), "exact", 9.0, 2048),
    ("qam64_exact", ("qam", 64), "exact", 15.0, 2048),
    ("shaped16_maxlog", ("shaped", 16), "maxlog", 10.0, 1024),
    ("shaped16_exact", ("shaped", 16), "exact", 10.0, 1024),
    ("psk8_maxlog", ("psk", 8), "maxlog", 11.0, 1024),
    ("psk8_exact", ("psk", 8), "exact", 11.0, 1024),
    ("cross32_exact", ("qam", 32), "exact", 14.0, 1024),
)
# (tag, code, method kind, method arguments, frames, LLR mean)
REGISTRY_LDPC_CASES = (
    ("codeA_ms", "A", "ms", {"max_iterations": 20}, 6, 2.2),
    ("dvbs2s_ms", "dvbs2s", "ms", {"scale": 0.75, "offset": 0.05, "max_iterations": 12}, 4, 1.8),
    ("dvbs2s_sp", "dvbs2s", "sp", {"max_iterations": 5}, 4, 0.8),
    ("pon_ms", "pon", "ms", {"max_iterations": 15, "early_stop": False}, 3, 3.0),
)


def registry_ldpc_llrs(frames: int, n: int, mean: float) -> np.ndarray:
    """Input LLRs of a recorded decode: ``mean + 1.5 N(0,1)`` of
    ``default_rng(70)``, the all-zero word."""
    rng = np.random.default_rng(70)
    return (mean + 1.5 * rng.standard_normal((frames, n))).astype(np.float32)


def _registry_constellation(Constellation, kind):
    family, order = kind
    if family == "qam":
        return Constellation.qam(order)
    if family == "psk":
        return Constellation.psk(order)
    return Constellation.qam(order).shaped(entropy=3.5)


def registry_case(ref: str) -> dict:
    """The reference's own launcher calls, recorded at its kernel registry:
    its ``compute_llr`` and ``decode`` run on stand-in CuPy arrays
    (:func:`_cupy_stand_in`) with recorders in place of the four launchers
    (:func:`_recording_registry`), so each recorded argument tuple is what the
    reference's host code builds for its CUDA kernels (tables from
    ``_device_tables``, ``inv_s2``, the schedule and the zero-padded
    posterior).  Beside each, the reference's CPU result for the same
    input, to compare the launchers' output with."""
    _import_reference(ref)
    cp = _cupy_stand_in()
    import commkit._cuda as cuda_module
    from commkit.coding import LDPCCode, MinSum, SumProduct, decode
    from commkit.mapping import Constellation, compute_llr

    from commkit_gb300 import workloads as W

    out = {}
    calls: list = []
    saved = _recording_registry(cuda_module, calls)
    try:
        for i, (tag, kind, method, esn0, n) in enumerate(REGISTRY_LLR_CASES):
            c = _registry_constellation(Constellation, kind)
            rng = np.random.default_rng(60 + i)
            idx = rng.integers(0, c.points.size, size=n)
            nv = float(c.power()) / 10 ** (esn0 / 10)
            noise = np.sqrt(nv / 2) * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
            x = (c.points[idx] + noise).astype(np.complex64)
            del calls[:]
            compute_llr(cp.view(x), esn0_db=esn0, constellation=c, method=method)
            assert len(calls) == 1, calls
            name, spec, args, kwargs = calls[0]
            out[f"{tag}_name"] = np.array(name)
            out[f"{tag}_x"] = args[0]
            for j, a in enumerate(args[1:]):
                if isinstance(a, tuple):
                    for t, arr in enumerate(a):
                        out[f"{tag}_arg{j}_{t}"] = arr
                    out[f"{tag}_arg{j}_len"] = np.int64(len(a))
                else:
                    out[f"{tag}_arg{j}"] = a
            out[f"{tag}_nargs"] = np.int64(len(args) - 1)
            for key, v in kwargs.items():
                out[f"{tag}_kw_{key}"] = np.asarray(v)
            out[f"{tag}_kwnames"] = np.array(sorted(kwargs))
            out[f"{tag}_esn0_db"] = np.float64(esn0)
            out[f"{tag}_want"] = np.asarray(
                compute_llr(x, esn0_db=esn0, constellation=c, method=method), np.float32).reshape(n, -1)  # fmt: skip
        for tag, which, kind, kw, frames, mean in REGISTRY_LDPC_CASES:
            if which == "A":
                code = LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
            elif which == "dvbs2s":
                code = LDPCCode.dvbs2("1/2", frame="short")
            else:
                code = LDPCCode.pon()
            method = MinSum(**kw) if kind == "ms" else SumProduct(**kw)
            llrs = registry_ldpc_llrs(frames, code.n, mean)
            del calls[:]
            decode(cp.view(llrs.reshape(-1)), code=code, method=method)
            assert len(calls) == 1, calls
            name, spec, args, kwargs = calls[0]
            out[f"{tag}_name"] = np.array(name)
            out[f"{tag}_sum_product"] = np.bool_(spec["sum_product"])
            # The posterior the reference builds (zeros, then the LLRs) is kept
            # as a digest: the tests rebuild it from registry_ldpc_llrs().
            assert np.array_equal(args[0][:, : code.n], llrs) and not args[0][:, code.n :].any()
            out[f"{tag}_app_digest"] = digest(args[0])
            out[f"{tag}_N"] = np.int64(args[0].shape[1])
            out[f"{tag}_row_ptr"], out[f"{tag}_cols"], out[f"{tag}_layer_ptr"] = args[1], args[2], args[3]
            for key, v in kwargs.items():
                out[f"{tag}_kw_{key}"] = np.asarray(v)
            out[f"{tag}_kwnames"] = np.array(sorted(kwargs))
            out[f"{tag}_n"] = np.int64(code.n)
            res = decode(llrs.reshape(-1), code=code, method=method)
            post = np.asarray(res.llrs, np.float32).reshape(frames, -1)
            if kind == "sp":
                out[f"{tag}_want_post"] = post
            else:
                out[f"{tag}_want_post_digest"] = digest(post)
                out[f"{tag}_want_post_first"] = post[0].copy()
            out[f"{tag}_want_iters"] = np.asarray(res.iterations, np.int32).reshape(-1)
            out[f"{tag}_want_valid"] = np.asarray(res.valid, bool).reshape(-1)
    finally:
        cuda_module._KERNEL_FACTORIES.update(saved)
    out["llr_tags"] = np.array([c[0] for c in REGISTRY_LLR_CASES])
    out["ldpc_tags"] = np.array([c[0] for c in REGISTRY_LDPC_CASES])
    return out


def main(ref: str, only: str | None = None) -> None:
    t0 = time.time()
    if only == "registry":
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as pool:
            res = pool.submit(registry_case, ref).result()
        np.savez_compressed(HERE / "registry_calls.npz", **res)
        print(f"registry fixtures written in {time.time() - t0:.0f} s")
        return
    if only == "wide":
        import multiprocessing as mp

        names = ("w64qc", "w64csr", "dvbs2n910")
        with ProcessPoolExecutor(max_workers=len(names), mp_context=mp.get_context("spawn")) as pool:
            parts = [f.result() for f in [pool.submit(wide_case, ref, nm) for nm in names]]
        wide = {}
        for part in parts:
            wide.update(part)
        np.savez_compressed(HERE / "ldpc_wide.npz", **wide)
        print(f"wide-row fixtures written in {time.time() - t0:.0f} s")
        return
    if only == "generator":
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as pool:
            res = pool.submit(generator_case, ref).result()
        np.savez_compressed(HERE / "ldpc_generator.npz", **res)
        print(f"generator fixtures written in {time.time() - t0:.0f} s")
        return
    if only == "api":
        import json
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as pool:
            res = pool.submit(api_signatures, ref).result()
        (HERE / "api_signatures.json").write_text(json.dumps(res, indent=1) + "\n")
        print(f"API signatures written in {time.time() - t0:.0f} s")
        return
    if only == "dvbs2":
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as pool:
            res = pool.submit(dvbs2_case, ref).result()
        np.savez_compressed(HERE / "dvbs2_normal.npz", **res)
        print(f"DVB-S2 fixtures written in {time.time() - t0:.0f} s")
        return
    if only == "gmi":
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as pool:
            res = pool.submit(gmi_case, ref).result()
        np.savez_compressed(HERE / "gmi_golden.npz", **res)
        print(f"GMI fixtures written in {time.time() - t0:.0f} s")
        return
    if only == "mpoint":
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as pool:
            res = pool.submit(mpoint_golden, ref).result()
        np.savez_compressed(HERE / "llr_mpoint_golden.npz", **res)
        print(f"M-point fixtures written in {time.time() - t0:.0f} s")
        return
    if only == "nonfinite":
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=2, mp_context=mp.get_context("spawn")) as pool:
            parts = [f.result() for f in [pool.submit(nonfinite_case, ref, w) for w in ("dvbs2s", "pon")]]
        np.savez_compressed(HERE / "ldpc_nonfinite.npz", **parts[0], **parts[1])
        print(f"non-finite fixtures written in {time.time() - t0:.0f} s")
        return
    if only == "sp":
        import multiprocessing as mp

        with ProcessPoolExecutor(max_workers=len(SP_CASES), mp_context=mp.get_context("spawn")) as pool:
            futs = [pool.submit(sp_case, ref, code, tag, mean, seed, frames, its)
                    for tag, code, mean, seed, frames, its in SP_CASES]
            parts = [f.result() for f in futs]
        sp = {}
        for part in parts:
            sp.update(part)
        np.savez_compressed(HERE / "ldpc_sp_golden.npz", **sp)
        print(f"sum-product fixtures written in {time.time() - t0:.0f} s")
        return
    jobs = {
        "qam": (qam_tables, (ref,)),
        "llr": (llr_golden, (ref,)),
        "A": (ldpc_qc_case, (ref, "A", 8, 4, 2.5, 20, "exact")),
        "B": (ldpc_qc_case, (ref, "B", 6, 16, 3.5, 20, "maxlog")),
        "C": (ldpc_qc_case, (ref, "C", 1, 16, 1.0, 50, "maxlog")),
        "dvbs2s": (kat_case, (ref, "dvbs2s")),
        "pon": (kat_case, (ref, "pon")),
    }
    import multiprocessing as mp

    with ProcessPoolExecutor(max_workers=len(jobs), mp_context=mp.get_context("spawn")) as pool:
        futs = {k: pool.submit(fn, *args) for k, (fn, args) in jobs.items()}
        res = {k: f.result() for k, f in futs.items()}
    np.savez_compressed(HERE / "qam_tables.npz", **res["qam"])
    np.savez_compressed(HERE / "llr_golden.npz", **res["llr"])
    ldpc = {}
    for k in ("A", "B", "C", "dvbs2s", "pon"):
        ldpc.update(res[k])
    np.savez_compressed(HERE / "ldpc_golden.npz", **ldpc)
    print(f"golden fixtures written in {time.time() - t0:.0f} s")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = next((a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")), None)
    if len(args) != 1:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_SOURCE_TREE [--only=PART]")
    main(args[0], only)
