"""Seeded synthetic workloads of the receiver back end (host-side, NumPy).

The codes and channels the benchmarks and tests run: seeded quasi-cyclic
base matrices (codes A, B and C), a host encoder for them, Gray-QAM
mapping, complex AWGN, and the batch builders of each measured
configuration.  All randomness is ``numpy.random.default_rng(seed)``, so a
workload is the same on every machine.  This is traffic generation, not
the decoder: inputs are made on the host, as the reference's own
``benchmarks/workloads.py`` makes them, then copied to the device.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# ---------------------------------------------------------------------------
# Base matrices
# ---------------------------------------------------------------------------


def dual_diagonal_base(mb: int, nb: int, z: int, info_weights, seed: int) -> np.ndarray:
    """A ``(mb, nb)`` QC base matrix with a dual-diagonal parity part.

    Columns ``nb - mb + j`` (the parity part) carry shift-0 identities at
    base rows ``j`` and ``j + 1``, so the lifted parity part is block lower
    bidiagonal with identities on its diagonal: invertible, and encoded by
    a block accumulation.  Info column ``c`` gets ``info_weights[c]``
    circulants at distinct random base rows with shifts uniform in
    ``[0, z)``.  Draws repeat (same generator) until every base row has at
    least one info circulant, so every check has >= 2 bits.
    """
    kb = nb - mb
    weights = np.asarray(info_weights, dtype=np.int64)
    if weights.size != kb or weights.min() < 1 or weights.max() > mb:
        raise ValueError("one weight in [1, mb] per info column")
    rng = np.random.default_rng(seed)
    while True:
        base = -np.ones((mb, nb), dtype=np.int64)
        for j in range(mb):
            base[j, kb + j] = 0
            if j + 1 < mb:
                base[j + 1, kb + j] = 0
        for c, w in enumerate(weights):
            rows = rng.choice(mb, size=int(w), replace=False)
            base[rows, c] = rng.integers(0, z, size=int(w))
        if np.all((base[:, :kb] >= 0).any(axis=1)):
            return base


@dataclass(frozen=True)
class QCSpec:
    name: str
    mb: int
    nb: int
    z: int
    seed: int
    info_weights: tuple[int, ...]

    def base(self) -> np.ndarray:
        return dual_diagonal_base(self.mb, self.nb, self.z, self.info_weights, self.seed)


def _spread(total: int, cols: int) -> tuple[int, ...]:
    q, r = divmod(total, cols)
    return tuple([q + 1] * r + [q] * (cols - r))


# Code A: 12 x 24, Z = 54 (N = 1296, K = 648, R = 1/2); info columns of
# weight 6 and 3, six of each; shifts from seed 0.
CODE_A = QCSpec("A", 12, 24, 54, 0, (6,) * 6 + (3,) * 6)
# Code B: 6 x 24, Z = 96 (N = 2304, K = 1728, R = 3/4); weight-3 info
# columns; seed 2.
CODE_B = QCSpec("B", 6, 24, 96, 2, (3,) * 18)
# Code C: 46 x 68, Z = 384 (N = 26112, K = 8448, R ~ 1/3); base density
# 0.1 (313 of 3128 entries: the 91 parity circulants and 222 info
# circulants spread evenly over the 22 info columns); seed 1.
CODE_C = QCSpec("C", 46, 68, 384, 1, _spread(round(0.1 * 46 * 68) - (2 * 46 - 1), 22))

CODES = {"A": CODE_A, "B": CODE_B, "C": CODE_C}


def lift(base: np.ndarray, z: int) -> tuple[np.ndarray, np.ndarray]:
    """``(checks, variables)`` of the lifted code, sorted by (row, column):
    entry ``s >= 0`` at ``(i, j)`` puts row ``i z + r`` on column
    ``j z + (r + s) mod z`` (the convention of ``LDPCCode.quasi_cyclic``,
    ``commkit/coding/ldpc.py:183-214``)."""
    bi, bj = np.nonzero(base >= 0)
    r = np.arange(z)
    rows = (bi[:, None] * z + r).ravel()
    cols = (bj[:, None] * z + (r + base[bi, bj][:, None]) % z).ravel()
    order = np.lexsort((cols, rows))
    return rows[order].astype(np.int32), cols[order].astype(np.int32)


# ---------------------------------------------------------------------------
# Encoding (block dual-diagonal parity)
# ---------------------------------------------------------------------------


def encode_qc(base: np.ndarray, z: int, info: np.ndarray) -> np.ndarray:
    """Systematic codewords ``[u | p]`` (int8, ``(F, N)``) of ``dual_diagonal_base`` codes.

    ``s = H_info u`` block by block (circulant ``s`` rolls the info block),
    then ``p_0 = s_0`` and ``p_b = s_b + p_{b-1}`` over GF(2).
    """
    mb, nb = base.shape
    kb = nb - mb
    info = np.asarray(info, dtype=np.int8)
    F = info.shape[0]
    u = info.reshape(F, kb, z)
    s = np.zeros((F, mb, z), dtype=np.int8)
    for i, j in zip(*np.nonzero(base[:, :kb] >= 0), strict=True):
        s[:, i, :] ^= np.roll(u[:, j, :], -int(base[i, j]), axis=1)
    p = np.bitwise_xor.accumulate(s, axis=1)
    return np.concatenate([info, p.reshape(F, mb * z)], axis=1)


def encode_accumulate(checks: np.ndarray, variables: np.ndarray, m: int, k: int,
                      info: np.ndarray) -> np.ndarray:  # fmt: skip
    """Systematic codewords ``[u | p]`` (int8, ``(F, k + m)``) of a code whose
    parity part is a staircase: check j holds parity bits k + j and, for
    j >= 1, k + j - 1 (DVB-S2's accumulator, ``commkit/coding/ldpc.py:217-236``).
    ``s = H_info u`` over GF(2), then ``p_j = p_{j-1} + s_j``."""
    from scipy.sparse import csr_matrix

    checks = np.asarray(checks, dtype=np.int64)
    variables = np.asarray(variables, dtype=np.int64)
    par = variables >= k
    j, c = checks[par], variables[par] - k
    if not np.all((c == j) | (c == j - 1)) or np.count_nonzero(c == j) != m:
        raise ValueError("the parity part is not a staircase")
    h_info = csr_matrix((np.ones(np.count_nonzero(~par), np.int32), (checks[~par], variables[~par])),
                        shape=(m, k))  # fmt: skip
    u = np.asarray(info, dtype=np.int8)
    s = (h_info @ u.T.astype(np.int32)).T % 2
    p = np.bitwise_xor.accumulate(s.astype(np.int8), axis=1)
    return np.concatenate([u, p], axis=1)


# ---------------------------------------------------------------------------
# Gray QAM and AWGN
# ---------------------------------------------------------------------------


def gray_qam_points(order: int) -> np.ndarray:
    """Unit-power Gray square QAM indexed by label (high half of the label
    on the in-phase axis), as ``commkit/mapping/gray.py:266-338`` builds it."""
    k = int(round(np.log2(order)))
    if 2**k != order or k % 2:
        raise ValueError(f"square QAM needs an even number of bits, got order {order}")
    n = k // 2
    L = 2**n
    gray = np.arange(L) ^ (np.arange(L) >> 1)
    pam = np.zeros(L)
    pam[gray] = np.linspace(-L + 1, L - 1, L)
    s = np.arange(order)
    pts = pam[s >> n] + 1j * pam[s & (L - 1)]
    return pts / np.sqrt(np.mean(np.abs(pts) ** 2))


def map_bits(bits: np.ndarray, order: int) -> np.ndarray:
    """Bits ``(..., n)`` (groups of k, MSB first) to complex64 symbols ``(..., n/k)``."""
    k = int(round(np.log2(order)))
    b = np.asarray(bits).reshape(*bits.shape[:-1], -1, k).astype(np.int64)
    label = (b << np.arange(k - 1, -1, -1)).sum(axis=-1)
    return gray_qam_points(order)[label].astype(np.complex64)


def awgn(symbols: np.ndarray, noise_var, rng: np.random.Generator) -> np.ndarray:
    """Circular complex Gaussian noise of variance ``noise_var`` (per frame
    when it is an array broadcasting against ``symbols``)."""
    nv = np.asarray(noise_var, dtype=np.float64)
    noise = rng.standard_normal(symbols.shape) + 1j * rng.standard_normal(symbols.shape)
    return (symbols + np.sqrt(nv / 2.0) * noise).astype(np.complex64)


def esn0_from_ebn0(ebn0_db, rate: float, bits_per_symbol: int):
    """Es/N0 = Eb/N0 + 10 log10(R k)."""
    return np.asarray(ebn0_db) + 10.0 * np.log10(rate * bits_per_symbol)


# ---------------------------------------------------------------------------
# Configurations
# ---------------------------------------------------------------------------


@dataclass
class CodedBatch:
    """Frames of one code through one channel: what a decode step eats."""

    spec: QCSpec
    base: np.ndarray
    order: int
    info: np.ndarray  # (F, K) int8
    symbols: np.ndarray  # (F, N / log2(order)) complex64
    noise_var: np.ndarray  # (F,) float64
    esn0_db: np.ndarray  # (F,)


def coded_batch(spec: QCSpec, frames: int, order: int, ebn0_db, seed: int) -> CodedBatch:
    """Random info bits -> encode -> Gray QAM -> AWGN at ``ebn0_db`` (scalar
    or one value per frame).  ``noise_var = 10^(-EsN0/10)`` for unit-power
    QAM."""
    base = spec.base()
    z = spec.z
    n_var = base.shape[1] * z
    kbits = (base.shape[1] - base.shape[0]) * z
    rng = np.random.default_rng(seed)
    info = rng.integers(0, 2, size=(frames, kbits), dtype=np.int8)
    words = encode_qc(base, z, info)
    k = int(round(np.log2(order)))
    if n_var % k:
        raise ValueError(f"N = {n_var} is not a multiple of {k} bits per symbol")
    tx = map_bits(words, order)
    esn0 = np.broadcast_to(
        esn0_from_ebn0(ebn0_db, kbits / n_var, k), (frames,)
    ).astype(np.float64)
    nv = 10.0 ** (-esn0 / 10.0)
    rx = awgn(tx, nv[:, None], rng)
    return CodedBatch(spec, base, order, info, rx, nv, esn0)


def demapper_batch(order: int, frames: int = 1024, frame_len: int = 4096, seed: int = 3,
                   esn0_range=(8.0, 20.0)):  # fmt: skip
    """Config 2: uniform random labels of Gray ``order``-QAM, per-frame Es/N0
    uniform in ``esn0_range`` dB; returns ``(rx (frames, frame_len), noise_var (frames,))``."""
    rng = np.random.default_rng(seed)
    k = int(round(np.log2(order)))
    bits = rng.integers(0, 2, size=(frames, frame_len * k), dtype=np.int8)
    tx = map_bits(bits, order)
    esn0 = rng.uniform(*esn0_range, size=frames)
    nv = 10.0 ** (-esn0 / 10.0)
    return awgn(tx, nv[:, None], rng), nv


# Eb/N0 (dB) where MinSum(max_iterations=50) decodes half the frames (FER
# ~ 0.5), measured with this package's decoder (bit-identical to the
# reference's) on 1024 frames (304 for C): code A on QPSK, B and C on 16-QAM.
WATERFALL_DB = {"A": 1.15, "B": 5.4, "C": 4.25}
MIXED_ORDERS = {"A": 4, "B": 16, "C": 16}


def mixed_workload(total: int = 8192, mix=(0.6, 0.3, 0.1), spread_db: float = 1.0, seed: int = 11):
    """Config 4: ``total`` frames of codes A/B/C in proportions ``mix``, each
    frame at an Eb/N0 uniform within +-``spread_db`` of its code's
    waterfall, so iteration counts spread from a few to the maximum.

    Returns ``{name: CodedBatch}`` for the codes with frames.
    """
    counts = np.floor(np.asarray(mix) * total).astype(int)
    counts[0] += total - counts.sum()
    rng = np.random.default_rng(seed)
    out = {}
    for (name, n), s in zip(zip(("A", "B", "C"), counts, strict=True), rng.integers(0, 2**31, 3), strict=True):
        if n <= 0:
            continue
        ebn0 = WATERFALL_DB[name] + rng.uniform(-spread_db, spread_db, size=int(n))
        out[name] = coded_batch(CODES[name], int(n), MIXED_ORDERS[name], ebn0, seed=int(s))
    return out
