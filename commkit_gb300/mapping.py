"""Soft-decision demapping: :class:`Constellation` and :func:`compute_llr`.

Mirrors ``commkit.mapping``: ``compute_llr`` (``commkit/mapping/llr.py:24-95``),
``Constellation`` with its factories (QAM square, rectangular and cross,
PSK, PAM, Maxwell-Boltzmann shaping) and ``Constellation.llr``
(``commkit/mapping/constellation.py:47-332``), and the GPU routing of
``commkit/mapping/_demap.py:150-352``.  Same signatures, same noise-variance
rules, same float32 ``inv_s2 = float32(1 / max(nv, 1e-20))``, same
``(..., N * k)`` output with each symbol's k bits adjacent, MSB first.
Separable square lattices take the per-axis kernels (max-log of a uniform
lattice in closed form, otherwise the level metrics with the axis priors);
every other constellation the M-point kernel; all on sm_103a
(``csrc/ck_llr*.cu``).

The device follows the data: CUDA input (a torch tensor or any
``__cuda_array_interface__`` array) gives CUDA output of the same library.
Host input raises ``TypeError``; there is no CPU path.
"""

from __future__ import annotations

import ctypes
import math
import warnings
from functools import cached_property
from typing import Any, NamedTuple

import numpy as np

from . import _device, _lib

__all__ = ["Constellation", "PrecisionWarning", "compute_llr", "compute_llr_frames", "inv_s2_frames"]


class PrecisionWarning(UserWarning):
    """Double-precision input reduced to float32 (``commkit/backend.py:38``)."""


class Axis(NamedTuple):
    """One axis of a separable constellation (``commkit/mapping/_lattice.py:24-30``)."""

    levels: np.ndarray  # (L,) ascending
    labels: np.ndarray  # (L, k_a) int8, MSB first
    pmf: np.ndarray | None
    bits: np.ndarray  # (k_a,) positions in the symbol label


def _gray(n: int) -> np.ndarray:
    """Binary-reflected Gray code of n bits: entry i is i ^ (i >> 1)."""
    i = np.arange(1 << n, dtype=np.int64)
    return i ^ (i >> 1)


def _gray_rank(n: int) -> np.ndarray:
    """Position of each n-bit Gray code word in the Gray sequence."""
    rank = np.empty(1 << n, dtype=np.int64)
    rank[_gray(n)] = np.arange(1 << n)
    return rank


def _ask_by_label(order: int, unipolar: bool = False) -> np.ndarray:
    """Gray ASK levels indexed by label: the j-th level from the bottom,
    -order + 1 + 2 j (shifted to start at 0 when unipolar), carries the
    label gray(j) (``commkit/mapping/gray.py:266-298``)."""
    k = int(np.log2(order))
    levels = -order + 1 + 2.0 * np.arange(order)
    if unipolar:
        levels = levels - levels.min()
    out = np.empty(order)
    out[_gray(k)] = levels
    return out


def _psk_by_label(order: int) -> np.ndarray:
    """Gray PSK on the unit circle indexed by label: phase 2 pi j / M carries
    gray(j); BPSK is real, -1 and +1 (``commkit/mapping/gray.py:227-263``)."""
    k = int(np.log2(order))
    if order == 2:
        return np.array([-1.0, 1.0])
    out = np.empty(order, dtype=complex)
    out[_gray(k)] = np.exp(2j * np.pi * np.arange(order) / order)
    return out


def _qam_by_label(order: int) -> np.ndarray:
    """Gray QAM indexed by label, before normalisation
    (``commkit/mapping/gray.py:142-151,301-425``): a square grid from two
    Gray ASK axes for even k (high half of the label on the in-phase axis);
    for 8 points a 4 x 2 rectangle (two MSBs in-phase); for other odd k a
    cross: the Gray rectangle of ceil(k/2) x floor(k/2) bits whose outer
    2^(ceil(k/2)-3) columns on each side are folded, rotated, onto the top
    and bottom of the central square."""
    k = int(np.log2(order))
    if order == 8:
        return (_ask_by_label(4)[:, None] + 1j * _ask_by_label(2)[None, :]).ravel()
    if k % 2 == 0:
        n = k // 2
        pam = _ask_by_label(1 << n)
        s = np.arange(order)
        return pam[s >> n] + 1j * pam[s & ((1 << n) - 1)]
    n_i, n_q = (k + 1) // 2, k // 2
    width, height = 1 << n_i, 1 << n_q
    s = np.arange(order)
    gi = _gray_rank(n_i)[s >> n_q]  # column of each label in the rectangle
    gq = _gray_rank(n_q)[s & ((1 << n_q) - 1)]  # row
    wing = (1 << (n_i - 3)) if n_i >= 3 else 0
    if wing:
        left, right = gi < wing, gi >= width - wing
        shift = (width - height) // 2
        col = np.where(left | right, gq + shift, gi)
        row = np.where(left, height + (wing - 1 - gi), gq)
        row = np.where(right, -1 - (gi - (width - wing)), row)
        gi, gq = col, row
    return (-width + 1 + 2.0 * gi) + 1j * (-height + 1 + 2.0 * gq)


def _unit_power(points: np.ndarray) -> np.ndarray:
    """Points over their RMS, the 2-norm over sqrt(M) as the reference computes
    it (``commkit/math.py:27-53,130-133``), so the points round identically."""
    return points / (np.linalg.norm(points) / np.sqrt(np.asarray(points.size, dtype=np.float64)))


def _entropy_bits(pmf: np.ndarray) -> float:
    p = pmf[pmf > 0]
    return float(-np.sum(p * np.log2(p)))


def _mb_pmf(energies: np.ndarray, nu: float) -> np.ndarray:
    """Maxwell-Boltzmann prior exp(-nu E) / Z (``commkit/mapping/shaping.py:169-185``)."""
    log_p = -nu * energies
    p = np.exp(log_p - log_p.max())
    return p / p.sum()


class Constellation:
    """Points with bit labels and an optional prior
    (``commkit/mapping/constellation.py:47-148``).

    ``points`` ``(M,)``, M a power of two >= 2, complex (two-dimensional) or
    real (PAM); ``bit_labels`` ``(M, k)`` MSB first, every pattern once
    (None: point i carries the bits of i); ``pmf`` the prior (None:
    uniform).  The factories put the point with label i at index i.
    """

    def __init__(self, points: Any, bit_labels: Any = None, pmf: Any = None, family: str | None = None):
        pts = np.asarray(points)
        if pts.ndim != 1 or pts.size < 2:
            raise ValueError(f"points must have shape (M,) with M >= 2, got {pts.shape}.")
        pts = pts.astype(np.complex128) if np.iscomplexobj(pts) else pts.astype(np.float64)
        if not np.all(np.isfinite(pts)):
            raise ValueError("points must be finite.")
        M = pts.size
        if np.unique(pts).size != M:
            raise ValueError("points must be distinct.")
        k = int(np.log2(M))
        if 2**k != M:
            raise ValueError(f"The number of points must be a power of 2, got {M}.")
        if bit_labels is None:
            labels = ((np.arange(M)[:, None] >> np.arange(k - 1, -1, -1)) & 1).astype(np.int8)
        else:
            labels = np.asarray(bit_labels)
            if labels.shape != (M, k):
                raise ValueError(f"bit_labels must have shape ({M}, {k}), got {labels.shape}.")
            if not np.all((labels == 0) | (labels == 1)):
                raise ValueError("bit_labels must contain only 0 and 1.")
            labels = labels.astype(np.int8)
            if np.unique(_packed(labels)).size != M:
                raise ValueError("bit_labels must assign every bit pattern once.")
        prior = None
        if pmf is not None:
            prior = np.asarray(pmf, dtype=np.float64)
            if prior.shape != (M,):
                raise ValueError(f"pmf must have shape ({M},), got {prior.shape}.")
            if not np.all(np.isfinite(prior)) or np.any(prior < 0):
                raise ValueError("pmf must be finite and non-negative.")
            total = prior.sum()
            if abs(total - 1.0) > 1e-6:
                raise ValueError(f"pmf must sum to 1, got {total:.8g}.")
            if abs(total - 1.0) > M * np.finfo(np.float64).eps:
                prior = prior / total
        if family is not None and family not in ("qam", "psk", "pam"):
            raise ValueError("family must be one of ('qam', 'psk', 'pam') or None.")
        for a in (pts, labels) + ((prior,) if prior is not None else ()):
            a.setflags(write=False)
        self.points, self.bit_labels, self.pmf, self.family = pts, labels, prior, family

    # -- factories ----------------------------------------------------------

    @classmethod
    def qam(cls, order: int) -> Constellation:
        """Gray M-QAM at unit average power: square for even log2 M, a 4 x 2
        rectangle for 8 points, cross for other odd log2 M."""
        return _named("qam", int(order), False)

    @classmethod
    def psk(cls, order: int) -> Constellation:
        """Gray M-PSK on the unit circle."""
        return _named("psk", int(order), False)

    @classmethod
    def pam(cls, order: int, *, unipolar: bool = False) -> Constellation:
        """Gray M-PAM (real) at unit average power; unipolar: non-negative levels."""
        return _named("pam", int(order), bool(unipolar))

    def shaped(self, *, nu: float | None = None, entropy: float | None = None) -> Constellation:
        """A copy with the Maxwell-Boltzmann prior P(s) ~ exp(-nu |s'|^2) (s'
        the points scaled to a minimum distance of 2), rescaled to unit power
        under the prior; exactly one of ``nu`` >= 0 and ``entropy`` (bits)
        (``commkit/mapping/constellation.py:179-210``)."""
        if (nu is None) == (entropy is None):
            raise ValueError("shaped() takes exactly one of nu or entropy.")
        energies = self._grid_energies()
        if np.ptp(energies) < 1e-9:
            raise ValueError("shaped() needs points of different energy; every point of "
                             "this constellation has the same energy.")  # fmt: skip
        if entropy is not None:
            nu = _nu_for_entropy(energies, float(entropy))
        if nu < 0:
            raise ValueError(f"nu must be >= 0, got {nu}.")
        pmf = _mb_pmf(energies, float(nu))
        scale = 1.0 / np.sqrt(np.dot(pmf, np.abs(self.points) ** 2))
        return Constellation(self.points * scale, self.bit_labels, pmf, self.family)

    def _grid_energies(self) -> np.ndarray:
        d = np.abs(self.points[:, None] - self.points[None, :])
        d_min = d[~np.eye(self.order, dtype=bool)].min()
        return np.abs(self.points * (2.0 / d_min)) ** 2

    # -- properties ---------------------------------------------------------

    @property
    def order(self) -> int:
        return int(self.points.size)

    @property
    def bits_per_symbol(self) -> int:
        return int(self.bit_labels.shape[1])

    @property
    def is_complex(self) -> bool:
        return bool(np.iscomplexobj(self.points))

    @property
    def entropy(self) -> float:
        """Entropy of the prior in bits per symbol (log2 M if uniform)."""
        return float(self.bits_per_symbol) if self.pmf is None else _entropy_bits(self.pmf)

    def power(self) -> float:
        """Average symbol power ``E[|s|^2]`` under the prior."""
        e = np.abs(self.points) ** 2
        return float(np.mean(e) if self.pmf is None else np.dot(self.pmf, e))

    def __repr__(self) -> str:
        shaped = "" if self.pmf is None else f", entropy={self.entropy:.4g}"
        return f"Constellation({self.family or 'custom'}, M={self.order}{shaped})"

    def __eq__(self, other: object) -> bool:
        if not isinstance(other, Constellation):
            return NotImplemented
        same_pmf = (self.pmf is None and other.pmf is None) or (
            self.pmf is not None and other.pmf is not None and np.array_equal(self.pmf, other.pmf))
        return (same_pmf and np.array_equal(self.points, other.points)
                and np.array_equal(self.bit_labels, other.bit_labels))  # fmt: skip

    def __hash__(self) -> int:
        h = self.__dict__.get("_hash")
        if h is None:
            h = self._hash = hash((self.points.tobytes(), self.bit_labels.tobytes(),
                                   None if self.pmf is None else self.pmf.tobytes()))  # fmt: skip
        return h

    # -- structure ----------------------------------------------------------

    @cached_property
    def _square_grid(self) -> tuple[float, float, int, np.ndarray] | None:
        """``(lowest level, step, side, lut)`` when the points fill a square
        lattice with the same levels on both axes, ``lut[i side + q]`` the
        point at level i in-phase and q in quadrature; else None
        (``commkit/mapping/_lattice.py:73-97``)."""
        side = int(round(self.order**0.5))
        if not self.is_complex or side * side != self.order or side < 2:
            return None
        re, im = self.points.real, self.points.imag
        lev_min = float(re.min())
        step = (float(re.max()) - lev_min) / (side - 1)
        if step <= 0 or abs(float(im.min()) - lev_min) > 1e-9 * step:
            return None
        gi, gq = (re - lev_min) / step, (im - lev_min) / step
        ri, rq = np.round(gi), np.round(gq)
        if max(np.abs(gi - ri).max(), np.abs(gq - rq).max()) > 1e-9:
            return None
        cell = ri.astype(np.int64) * side + rq.astype(np.int64)
        if cell.min() < 0 or cell.max() >= self.order or np.unique(cell).size != self.order:
            return None
        lut = np.empty(self.order, dtype=np.int64)
        lut[cell] = np.arange(self.order)
        return lev_min, step, side, lut

    @cached_property
    def _axes(self) -> tuple[Axis, Axis] | None:
        """Per-axis levels, labels, marginal prior and bit positions when the
        square lattice factors into two axes (every bit constant along one
        axis, the prior a product of marginals), else None
        (``commkit/mapping/_lattice.py:100-124``)."""
        grid = self._square_grid
        if grid is None:
            return None
        side, lut = grid[2], grid[3]
        lab = self.bit_labels[lut].reshape(side, side, -1)  # [in-phase level, quadrature level, bit]
        on_re = np.all(lab == lab[:, :1, :], axis=(0, 1))
        on_im = np.all(lab == lab[:1, :, :], axis=(0, 1))
        if not np.all(on_re ^ on_im):
            return None
        bits_re, bits_im = np.flatnonzero(on_re), np.flatnonzero(on_im)
        if 2**bits_re.size != side or 2**bits_im.size != side:
            return None
        grid_pts = self.points[lut].reshape(side, side)
        pmf_re = pmf_im = None
        if self.pmf is not None:
            joint = self.pmf[lut].reshape(side, side)
            pmf_re, pmf_im = joint.sum(axis=1), joint.sum(axis=0)
            if not np.allclose(joint, np.outer(pmf_re, pmf_im), rtol=1e-9, atol=0.0):
                return None
        return (Axis(grid_pts[:, 0].real, lab[:, 0][:, bits_re], pmf_re, bits_re),
                Axis(grid_pts[0, :].imag, lab[0, :][:, bits_im], pmf_im, bits_im))  # fmt: skip

    def llr(self, symbols: Any, *, noise_var: float, method: str = "maxlog") -> Any:
        """Bit LLRs (positive: bit 0 more likely), ``float32 (..., N * k)``
        on the symbols' device (``commkit/mapping/constellation.py:309-332``):
        separable lattices per axis, every other constellation over all its
        points."""
        out = _calls_llr(symbols, noise_var, self, method)
        if out is not None:
            return out
        nv = _finite(noise_var, "Constellation.llr(): noise_var", low=0.0)
        return self._llr(symbols, _device.wrap(symbols, "symbols"), nv, method)

    def _llr(self, symbols: Any, x: _device.DeviceArray, nv: float, method: str) -> Any:
        """``llr`` on already wrapped symbols (``compute_llr`` wraps once)."""
        if x.dtype.kind != "c":
            # Real noise of variance s2: the in-phase part of circular noise of 2 s2.
            nv = 2.0 * nv
        if self._axes is not None:
            return _llr_separable_gpu(symbols, x, self, nv, method)
        return _llr_points_gpu(symbols, x, self, nv, method)


def _nu_for_entropy(energies: np.ndarray, entropy: float) -> float:
    """The nu whose Maxwell-Boltzmann prior has ``entropy`` bits, by Brent's
    method on [0, nu_hi] (``commkit/mapping/shaping.py:188-214``)."""
    from scipy.optimize import brentq

    min_e = float(energies.min())
    m_min = int(np.count_nonzero(np.isclose(energies, min_e, rtol=1e-9, atol=1e-12)))
    min_h, max_h = float(np.log2(m_min)), float(np.log2(energies.size))
    if not np.isfinite(entropy) or not min_h < entropy <= max_h:
        raise ValueError(f"entropy must be in ({min_h:g}, {max_h:g}] bits, got {entropy}.")
    if np.isclose(entropy, max_h, atol=1e-8):
        return 0.0

    def gap(nu: float) -> float:
        return _entropy_bits(_mb_pmf(energies, nu)) - entropy

    nu_hi = 0.01
    while gap(nu_hi) > 0:
        nu_hi *= 10.0
    return float(brentq(gap, 0.0, nu_hi, xtol=1e-12, rtol=1e-12))


_NAMED: dict[tuple[str, int, bool], Constellation] = {}


def _named(family: str, order: int, unipolar: bool) -> Constellation:
    key = (family, order, unipolar)
    c = _NAMED.get(key)
    if c is None:
        if order < 2 or order & (order - 1):
            raise ValueError(f"order must be a power of 2 >= 2, got {order}.")
        if family == "psk":
            pts = _psk_by_label(order)
        elif family == "pam":
            pts = _unit_power(_ask_by_label(order, unipolar))
        else:
            pts = _unit_power(_qam_by_label(order))
        c = _NAMED[key] = Constellation(pts, family=family)
    return c


def _qam(order: int) -> Constellation:
    return Constellation.qam(order)


def _finite(v: float, name: str, low: float | None = None) -> float:
    f = float(v)
    if not math.isfinite(f):
        raise ValueError(f"{name} must be finite, got {v!r}")
    if low is not None and f < low:
        raise ValueError(f"{name} must be >= {low}, got {v!r}")
    return f


def _noise_variance(noise_var, esn0_db, constellation: Constellation, real: bool, fn: str) -> float:
    """``commkit/mapping/_demap.py:48-68``: ``N0 = Es / 10^(EsN0/10)``, halved for real symbols."""
    if (noise_var is None) == (esn0_db is None):
        raise ValueError(f"{fn}: give one of noise_var and esn0_db.")
    if noise_var is not None:
        return _finite(noise_var, f"{fn}: noise_var", low=0.0)
    snr = _finite(esn0_db, f"{fn}: esn0_db")
    n0 = constellation.power() / 10 ** (snr / 10)
    return n0 / 2 if real else n0


def _calls_llr(symbols: Any, noise_var: Any, c: Any, method: Any) -> Any:
    """The per-call extension's demap of a form an earlier call registered
    (complex64 torch symbols, contiguous, a float noise variance); None when
    it does not take the call and the general path has to."""
    per = getattr(c, "_calls_llr", None)
    if per is None or not isinstance(method, str):
        return None
    entries = per.get(method)
    if entries is None:
        return None
    out = _lib.calls().llr(symbols, noise_var, entries)
    if out.__class__ is int:
        _lib.check(out, "compute_llr()")
    return out


def _register_calls(c: Constellation, method: str, device: int, entry: tuple) -> None:
    """Lets later calls of ``c`` and ``method`` on ``device`` go straight to
    the per-call extension: ``entry`` = (kind, exact, three table addresses,
    M, k), kind 0 the closed-form max-log, 1 the per-axis levels, 2 every
    point; kept per method in a list indexed by device."""
    if _lib.calls() is None:
        return
    per = c.__dict__.setdefault("_calls_llr", {})
    entries = per.get(method) or []
    if len(entries) <= device:
        entries = entries + [None] * (device + 1 - len(entries))
    entries[device] = entry
    per[method] = entries


def inv_s2(noise_var: float) -> float:
    """``float(float32(1 / max(nv, 1e-20)))`` (``commkit/mapping/_demap.py:312``)."""
    return float(np.float32(1.0 / max(float(noise_var), 1e-20)))


def _check_method(method: str) -> None:
    if method not in ("maxlog", "exact"):
        raise ValueError(f"Unknown method: {method}. Use 'maxlog' or 'exact'.")


# ---------------------------------------------------------------------------
# Device tables (``commkit/backend.py:265-287``: per owner, kind and device)
# ---------------------------------------------------------------------------



def _opposite_levels(labels: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """For each bit b and level s of an axis, the nearest level below
    (``lo[b, s]``) and above (``hi[b, s]``) whose bit b differs from level
    s's, -1 where there is none: ``(k_a, L)`` int32, the closed-form
    max-log's opposite levels (``commkit/mapping/_demap.py:82-106``).

    One upward and one downward scan per bit: when a level's bit equals the
    bit of the level just below it, both share their nearest differing
    level below; otherwise that is the level just below (and likewise
    upwards)."""
    L, k = labels.shape
    lo = np.full((k, L), -1, np.int32)
    hi = np.full((k, L), -1, np.int32)
    for b in range(k):
        bit = labels[:, b]
        for s in range(1, L):
            lo[b, s] = s - 1 if bit[s] != bit[s - 1] else lo[b, s - 1]
        for s in range(L - 2, -1, -1):
            hi[b, s] = s + 1 if bit[s] != bit[s + 1] else hi[b, s + 1]
    return lo, hi


def _packed(labels: np.ndarray) -> np.ndarray:
    k = labels.shape[1]
    return (labels.astype(np.int64) << np.arange(k - 1, -1, -1)).sum(axis=1).astype(np.int32)


def _log_prior(pmf: np.ndarray | None, size: int) -> np.ndarray:
    """float32 log prior, zeros for none (``commkit/mapping/_demap.py:125-129``)."""
    if pmf is None:
        return np.zeros(size, dtype=np.float32)
    return np.log(np.clip(np.asarray(pmf, np.float64), 1e-40, None)).astype(np.float32)


def host_tables(constellation: Constellation, kind: str) -> tuple[np.ndarray, ...]:
    """Host tables in the reference launchers' tuple layouts:
    ``"maxlog"``: (levels f32, labels i32, lo, hi, positions i32) per axis;
    ``"levels"``: (levels f32, log prior f32, labels i32, positions i32) per axis;
    ``"points"``: (points c64, log prior f32, labels i32) of every point."""
    if kind == "points":
        c = constellation
        return (c.points.astype(np.complex64), _log_prior(c.pmf, c.order), _packed(c.bit_labels))
    out: list[np.ndarray] = []
    for a in constellation._axes:
        if kind == "maxlog":
            lo, hi = _opposite_levels(a.labels)
            out += [a.levels.astype(np.float32), _packed(a.labels), lo, hi, a.bits.astype(np.int32)]
        else:
            out += [a.levels.astype(np.float32), _log_prior(a.pmf, a.levels.size),
                    _packed(a.labels), a.bits.astype(np.int32)]  # fmt: skip
    return tuple(out)


def _table_kind(c: Constellation, method: str) -> str:
    """Which kernel serves ``c`` (``commkit/mapping/_demap.py:112-118,
    298-352``, ``constellation.py:327-332``): the closed form for max-log of
    a uniform separable lattice, the per-axis level metrics for other
    separable lattices, every point otherwise.  Remembered on the
    (immutable) instance per method."""
    memo = c.__dict__.get("_table_kinds")
    if memo is None:
        memo = c.__dict__["_table_kinds"] = {}
    kind = memo.get(method)
    if kind is None:
        if c._axes is None:
            kind = "points"
        elif method == "maxlog" and all(a.pmf is None and a.levels.size >= 2 for a in c._axes):
            kind = "maxlog"
        else:
            kind = "levels"
        memo[method] = kind
    return kind


def device_tables(constellation: Constellation, kind: str, like: _device.DeviceArray):
    # Kept on the (immutable) instance: a lookup by value would compare the
    # points on every call.
    per = constellation.__dict__.get("_device_tables")
    if per is None:
        per = constellation.__dict__["_device_tables"] = {}
    key = (kind, like.device)
    t = per.get(key)
    if t is None:
        import torch

        dev = torch.device("cuda", like.device)
        t = per[key] = tuple(torch.from_numpy(a.copy()).to(dev) for a in host_tables(constellation, kind))
    return t


def _axis_args(constellation: Constellation, kind: str, like: _device.DeviceArray) -> tuple:
    """The two axes' C-ABI structs of ``device_tables`` and pointers to them
    (``ctypes.byref``), built once per table kind and device and kept with
    the tables, so a call passes them as they are."""
    per = constellation.__dict__.get("_axis_args")
    if per is None:
        per = constellation.__dict__["_axis_args"] = {}
    key = (kind, like.device)
    args = per.get(key)
    if args is None:
        tables = device_tables(constellation, kind, like)
        half = len(tables) // 2
        re, im = _axis_struct(tables[:half], kind), _axis_struct(tables[half:], kind)
        args = per[key] = (re, im, ctypes.byref(re), ctypes.byref(im), tables)
    return args


def _axis_struct(tables, kind: str):
    if kind == "maxlog":
        lev, lab, lo, hi, pos = tables
        return _lib.AxisMaxlog(lev.data_ptr(), lab.data_ptr(), lo.data_ptr(), hi.data_ptr(),
                               pos.data_ptr(), lev.numel(), pos.numel())  # fmt: skip
    lev, logp, lab, pos = tables
    return _lib.AxisLevels(lev.data_ptr(), logp.data_ptr(), lab.data_ptr(), pos.data_ptr(),
                           lev.numel(), pos.numel())  # fmt: skip


# ---------------------------------------------------------------------------
# LLRs
# ---------------------------------------------------------------------------


def _as_complex64(symbols: Any, x: _device.DeviceArray, fn: str):
    """complex64 flat view (a copy for other dtypes), as ``astype(complex64)``."""
    if x.dtype == np.complex128:
        warnings.warn(f"{fn}: complex128 input computed in float32", PrecisionWarning, stacklevel=4)
    if x.kind == "torch":
        import torch

        t = symbols.reshape(-1)
        if t.dtype != torch.complex64:
            t = t.to(torch.complex64)
        return t.contiguous()
    import cupy

    return cupy.ascontiguousarray(symbols.reshape(-1).astype(cupy.complex64))


def _llr_separable_gpu(symbols: Any, x: _device.DeviceArray, c: Constellation, nv: float,
                       method: str) -> Any:  # fmt: skip
    """``commkit/mapping/_demap.py:298-352`` on the sm_103a kernels."""
    _check_method(method)
    k = c.bits_per_symbol
    if x.kind == "torch" and x.contiguous and x.dtype == np.complex64:
        # The common case: the symbols as they are, no copy and no new wrap.
        ptr, n = x.ptr, x.size
    else:
        flat = _as_complex64(symbols, x, "compute_llr() / Constellation.llr()")
        fx = _device.wrap(flat, "symbols")
        ptr, n = fx.ptr, fx.size
    if n >= 2**31:
        raise ValueError(f"at most 2**31 - 1 symbols per call, got {n}")
    # The output in its final shape, (..., N * k): the same memory as (n, k).
    shape = tuple(x.shape[:-1]) + (x.shape[-1] * k,) if x.ndim else (k,)
    if x.kind == "torch":
        torch = _device._torch()
        out = torch.empty(shape, dtype=torch.float32, device=symbols.device)
        out_ptr = out.data_ptr()
    else:
        out = _device.empty(x, shape, np.float32)
        out_ptr = _device.wrap(out, "out").ptr
    kind = _table_kind(c, method)
    with _device.on_device(x):
        _, _, re_ref, im_ref, _ = _axis_args(c, kind, x)
        stream = _device.stream_of(x)
        lib = _lib.lib()
        if kind == "maxlog":
            st = lib.ck_llr_separable_maxlog(ptr, n, re_ref, im_ref, inv_s2(nv), out_ptr, stream)
        else:
            st = lib.ck_llr_separable(ptr, n, re_ref, im_ref, inv_s2(nv), 1 if method == "exact" else 0,
                                      out_ptr, stream)  # fmt: skip
        _lib.check(st, "compute_llr()")
    if x.kind == "torch" and x.contiguous and x.dtype == np.complex64:
        re, im = _axis_args(c, kind, x)[:2]
        _register_calls(c, method, x.device, (0 if kind == "maxlog" else 1, 1 if method == "exact" else 0,
                                              ctypes.addressof(re), ctypes.addressof(im), 0, 0, k))  # fmt: skip
    return out


def _llr_points_gpu(symbols: Any, x: _device.DeviceArray, c: Constellation, nv: float,
                    method: str) -> Any:  # fmt: skip
    """``commkit/mapping/_demap.py:150-219`` (the GPU branch) on the
    sm_103a M-point kernel."""
    _check_method(method)
    k = c.bits_per_symbol
    if k > _lib.CK_LLR_MAX_K:
        raise ValueError(f"compute_llr(): GPU input supports at most {_lib.CK_LLR_MAX_K} bits "
                         f"per symbol, the constellation has {k}")  # fmt: skip
    flat = _as_complex64(symbols, x, "compute_llr() / Constellation.llr()")
    fx = _device.wrap(flat, "symbols")
    n = fx.size
    if n >= 2**31:
        raise ValueError(f"at most 2**31 - 1 symbols per call, got {n}")
    out = _device.empty(x, (n, k), np.float32)
    od = _device.wrap(out, "out")
    with _device.on_device(x):
        pts, logp, lab = device_tables(c, "points", x)
        st = _lib.lib().ck_llr_points(fx.ptr, n, pts.data_ptr(), logp.data_ptr(), lab.data_ptr(),
                                      c.order, k, inv_s2(nv), 1 if method == "exact" else 0, od.ptr,
                                      _device.stream_of(x))  # fmt: skip
        _lib.check(st, "compute_llr()")
    if x.kind == "torch" and x.contiguous and x.dtype == np.complex64:
        _register_calls(c, method, x.device, (2, 1 if method == "exact" else 0, pts.data_ptr(), logp.data_ptr(),
                                              lab.data_ptr(), c.order, k))  # fmt: skip
    shape = tuple(x.shape[:-1]) + (x.shape[-1] * k,) if x.ndim else (k,)
    return out.reshape(shape)


def compute_llr(symbols: Any, *, noise_var: float | None = None, esn0_db: float | None = None,
                constellation: Constellation | None = None, method: str = "maxlog") -> Any:  # fmt: skip
    """Bit LLRs of received symbols (``commkit/mapping/llr.py:24-95``).

    ``symbols`` ``(..., N)`` on a CUDA device; one of ``noise_var`` (the
    variance ``E|n|^2`` of the noise in the symbols) and ``esn0_db``;
    ``method`` ``"maxlog"`` or ``"exact"``.  Returns float32 ``(..., N * k)``
    on the symbols' device, the k bits of a symbol adjacent, MSB first.
    """
    if esn0_db is None:
        out = _calls_llr(symbols, noise_var, constellation, method)
        if out is not None:
            return out
    if constellation is None:
        raise ValueError("compute_llr(): constellation is required for array input.")
    x = _device.wrap(symbols, "symbols")
    nv = _noise_variance(noise_var, esn0_db, constellation, x.dtype.kind != "c", "compute_llr()")
    return constellation._llr(symbols, x, nv, method)


def inv_s2_frames(noise_var: Any) -> np.ndarray:
    """Per-frame ``float32(1 / max(nv, 1e-20))``, as :func:`inv_s2` for each frame."""
    nv = np.asarray(noise_var, dtype=np.float64).reshape(-1)
    if not np.all(np.isfinite(nv)) or np.any(nv < 0):
        raise ValueError("noise_var must be finite and >= 0")
    return (1.0 / np.maximum(nv, 1e-20)).astype(np.float32)


def compute_llr_frames(symbols: Any, *, noise_var: Any = None, constellation: Constellation,
                       method: str = "maxlog", inv_s2: Any = None, out: Any = None) -> Any:  # fmt: skip
    """Batched demapping with one noise variance per frame (an extension).

    ``symbols`` ``(F, S)`` complex64 on a CUDA device, ``noise_var`` ``(F,)``
    (host array or sequence).  Returns ``(F, S * k)`` float32; row ``f``
    equals ``compute_llr(symbols[f], noise_var=noise_var[f], ...)`` bit for
    bit, in one launch instead of F.  Instead of ``noise_var``, ``inv_s2``
    may give the per-frame ``float32(1 / max(nv, 1e-20))`` already on the
    device (:func:`inv_s2_frames`), and ``out`` a preallocated output; with
    both, the call does no host-to-device copy and no allocation, so it can
    be captured in a CUDA graph.
    """
    _check_method(method)
    x = _device.wrap(symbols, "symbols")
    _device.check(x, "symbols", np.complex64, (None, None))
    F, S = x.shape
    k = constellation.bits_per_symbol
    if (noise_var is None) == (inv_s2 is None):
        raise ValueError("compute_llr_frames(): give one of noise_var and inv_s2.")
    s2_host = None
    if inv_s2 is None:
        s2_host = inv_s2_frames(noise_var)
        if s2_host.size != F:
            raise ValueError(f"noise_var needs one value per frame ({F}), got {s2_host.size}")
    if out is None:
        out = _device.empty(x, (F, S * k), np.float32)
    od = _device.wrap(out, "out")
    _device.check(od, "out", np.float32, (F, S * k))
    if F * S == 0:
        return out
    kind = _table_kind(constellation, method)
    with _device.on_device(x):
        s2 = _device.to_device(x, s2_host) if s2_host is not None else inv_s2
        sd = _device.wrap(s2, "inv_s2")
        _device.check(sd, "inv_s2", np.float32, (F,))
        tables = device_tables(constellation, kind, x)
        stream = _device.stream_of(x)
        lib = _lib.lib()
        if kind == "points":
            pts, logp, lab = tables
            st = lib.ck_llr_points_frames(x.ptr, F * S, S, sd.ptr, pts.data_ptr(), logp.data_ptr(),
                                          lab.data_ptr(), constellation.order, k,
                                          1 if method == "exact" else 0, od.ptr, stream)  # fmt: skip
            _lib.check(st, "compute_llr_frames()")
            return out
        half = len(tables) // 2
        re, im = _axis_struct(tables[:half], kind), _axis_struct(tables[half:], kind)
        if kind == "maxlog":
            st = lib.ck_llr_separable_maxlog_frames(x.ptr, F * S, S, sd.ptr, ctypes.byref(re),
                                                    ctypes.byref(im), od.ptr, stream)  # fmt: skip
        else:
            st = lib.ck_llr_separable_frames(x.ptr, F * S, S, sd.ptr, ctypes.byref(re),
                                             ctypes.byref(im), 1 if method == "exact" else 0,
                                             od.ptr, stream)  # fmt: skip
        _lib.check(st, "compute_llr_frames()")
    return out
