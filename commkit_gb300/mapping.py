"""Soft-decision demapping: :class:`Constellation` and :func:`compute_llr`.

Mirrors ``commkit.mapping`` for the separable constellations (Gray square
QAM, QPSK included): ``compute_llr`` (``commkit/mapping/llr.py:24-95``),
``Constellation.llr`` (``commkit/mapping/constellation.py:309-332``) and the
GPU routing of ``commkit/mapping/_demap.py:298-352``.  Same signatures, same
noise-variance rules, same float32 ``inv_s2 = float32(1 / max(nv, 1e-20))``,
same ``(..., N * k)`` output with each symbol's k bits adjacent, MSB first.
Max-log takes the closed form, exact the level metrics, both on the
sm_103a kernels of ``csrc/ck_llr*.cu``.

The device follows the data: CUDA input (a torch tensor or any
``__cuda_array_interface__`` array) gives CUDA output of the same library.
Host input raises ``TypeError``; there is no CPU path.
"""

from __future__ import annotations

import ctypes
import warnings
import weakref
from functools import cached_property
from typing import Any, NamedTuple

import numpy as np

from . import _device, _lib
from .workloads import gray_qam_points

__all__ = ["Constellation", "PrecisionWarning", "compute_llr", "compute_llr_frames", "inv_s2_frames"]


class PrecisionWarning(UserWarning):
    """Double-precision input reduced to float32 (``commkit/backend.py:38``)."""


class Axis(NamedTuple):
    """One axis of a separable constellation (``commkit/mapping/_lattice.py:24-30``)."""

    levels: np.ndarray  # (L,) ascending
    labels: np.ndarray  # (L, k_a) int8, MSB first
    pmf: np.ndarray | None
    bits: np.ndarray  # (k_a,) positions in the symbol label


class Constellation:
    """Gray square QAM, the separable constellations of the demapper.

    ``points[i]`` is the point whose label is the binary value of ``i``
    (``commkit/mapping/gray.py:99-162``); ``bit_labels`` the labels, MSB
    first.  Value semantics: equal orders compare equal.
    """

    def __init__(self, order: int):
        self.order = int(order)
        self.points = gray_qam_points(self.order)
        k = int(round(np.log2(self.order)))
        self.bits_per_symbol = k
        idx = np.arange(self.order)
        self.bit_labels = ((idx[:, None] >> np.arange(k - 1, -1, -1)) & 1).astype(np.int8)
        self.pmf = None

    @classmethod
    def qam(cls, order: int) -> Constellation:
        """Gray-labeled square M-QAM at unit average power (even ``log2 M``)."""
        return _qam(int(order))

    def __repr__(self) -> str:
        return f"Constellation.qam({self.order})"

    def __eq__(self, other: object) -> bool:
        return isinstance(other, Constellation) and other.order == self.order

    def __hash__(self) -> int:
        return hash(("qam", self.order))

    def power(self) -> float:
        """Average symbol power ``E[|s|^2]``."""
        return float(np.mean(np.abs(self.points) ** 2))

    @cached_property
    def _axes(self) -> tuple[Axis, Axis]:
        """Per-axis levels, labels and bit positions (``_lattice.py:100-124``).

        Level ``i`` of either axis (ascending) carries the axis label
        ``gray(i)``; the in-phase axis holds the label's high half.
        """
        k = self.bits_per_symbol
        ka = k // 2
        L = 1 << ka
        gray = np.arange(L) ^ (np.arange(L) >> 1)
        labels = ((gray[:, None] >> np.arange(ka - 1, -1, -1)) & 1).astype(np.int8)
        axes = []
        for bits, part in ((np.arange(ka), np.real), (np.arange(ka, k), np.imag)):
            shift = k - 1 - int(bits[-1])
            axis_label = (np.arange(self.order) >> shift) & (L - 1)
            levels = np.array([part(self.points[np.flatnonzero(axis_label == g)[0]]) for g in gray])
            axes.append(Axis(levels, labels, None, bits))
        return tuple(axes)  # type: ignore[return-value]

    def llr(self, symbols: Any, *, noise_var: float, method: str = "maxlog") -> Any:
        """Bit LLRs (positive: bit 0 more likely), ``float32 (..., N * k)``
        on the symbols' device (``commkit/mapping/constellation.py:309-332``)."""
        nv = _finite(noise_var, "Constellation.llr(): noise_var", low=0.0)
        x = _device.wrap(symbols, "symbols")
        if x.dtype.kind != "c":
            # Real noise of variance s2: the in-phase part of circular noise of 2 s2.
            nv = 2.0 * nv
        return _llr_separable_gpu(symbols, x, self, nv, method)


_QAM_CACHE: dict[int, Constellation] = {}


def _qam(order: int) -> Constellation:
    c = _QAM_CACHE.get(order)
    if c is None:
        c = _QAM_CACHE[order] = Constellation(order)
    return c


def _finite(v: float, name: str, low: float | None = None) -> float:
    f = float(v)
    if not np.isfinite(f):
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


def inv_s2(noise_var: float) -> float:
    """``float(float32(1 / max(nv, 1e-20)))`` (``commkit/mapping/_demap.py:312``)."""
    return float(np.float32(1.0 / max(float(noise_var), 1e-20)))


def _check_method(method: str) -> None:
    if method not in ("maxlog", "exact"):
        raise ValueError(f"Unknown method: {method}. Use 'maxlog' or 'exact'.")


# ---------------------------------------------------------------------------
# Device tables (``commkit/backend.py:265-287``: per owner, kind and device)
# ---------------------------------------------------------------------------

_TABLES: weakref.WeakKeyDictionary = weakref.WeakKeyDictionary()


def _opposite_levels(labels: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """``lo``/``hi`` ``(k_a, L)`` int32 (``commkit/mapping/_demap.py:82-106``):
    the nearest level below / above with the other bit value, -1 for none."""
    L, k = labels.shape
    lo = np.empty((k, L), np.int32)
    hi = np.empty((k, L), np.int32)
    for b in range(k):
        col = labels[:, b]
        change = col[1:] != col[:-1]
        run = np.concatenate([[0], np.cumsum(change)])
        starts = np.concatenate([[0], np.flatnonzero(change) + 1])
        ends = np.concatenate([np.flatnonzero(change), [L - 1]])
        lo[b] = starts[run] - 1
        hi[b] = np.where(ends[run] + 1 < L, ends[run] + 1, -1)
    return lo, hi


def _packed(labels: np.ndarray) -> np.ndarray:
    k = labels.shape[1]
    return (labels.astype(np.int64) << np.arange(k - 1, -1, -1)).sum(axis=1).astype(np.int32)


def host_tables(constellation: Constellation, kind: str) -> tuple[np.ndarray, ...]:
    """Host tables per axis, in the reference launchers' tuple layouts:
    ``"maxlog"``: (levels f32, labels i32, lo, hi, positions i32) x 2;
    ``"levels"``: (levels f32, log prior f32, labels i32, positions i32) x 2."""
    out: list[np.ndarray] = []
    for a in constellation._axes:
        if kind == "maxlog":
            lo, hi = _opposite_levels(a.labels)
            out += [a.levels.astype(np.float32), _packed(a.labels), lo, hi, a.bits.astype(np.int32)]
        else:
            out += [a.levels.astype(np.float32), np.zeros(a.levels.size, np.float32),
                    _packed(a.labels), a.bits.astype(np.int32)]  # fmt: skip
    return tuple(out)


def device_tables(constellation: Constellation, kind: str, like: _device.DeviceArray):
    per = _TABLES.setdefault(constellation, {})
    key = (kind, like.device)
    t = per.get(key)
    if t is None:
        import torch

        dev = torch.device("cuda", like.device)
        t = per[key] = tuple(torch.from_numpy(a.copy()).to(dev) for a in host_tables(constellation, kind))
    return t


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
    flat = _as_complex64(symbols, x, "compute_llr() / Constellation.llr()")
    fx = _device.wrap(flat, "symbols")
    n = fx.size
    if n >= 2**31:
        raise ValueError(f"at most 2**31 - 1 symbols per call, got {n}")
    out = _device.empty(x, (n, k), np.float32)
    od = _device.wrap(out, "out")
    kind = "maxlog" if method == "maxlog" else "levels"
    with _device.on_device(x):
        tables = device_tables(c, kind, x)
        half = len(tables) // 2
        re, im = _axis_struct(tables[:half], kind), _axis_struct(tables[half:], kind)
        stream = _device.stream_of(x)
        lib = _lib.lib()
        if kind == "maxlog":
            st = lib.ck_llr_separable_maxlog(fx.ptr, n, ctypes.byref(re), ctypes.byref(im),
                                             inv_s2(nv), od.ptr, stream)  # fmt: skip
        else:
            st = lib.ck_llr_separable(fx.ptr, n, ctypes.byref(re), ctypes.byref(im), inv_s2(nv),
                                      1 if method == "exact" else 0, od.ptr, stream)  # fmt: skip
        _lib.check(st, "compute_llr()")
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
    if constellation is None:
        raise ValueError("compute_llr(): constellation is required for array input.")
    x = _device.wrap(symbols, "symbols")
    nv = _noise_variance(noise_var, esn0_db, constellation, x.dtype.kind != "c", "compute_llr()")
    return constellation.llr(symbols, noise_var=nv, method=method)


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
    kind = "maxlog" if method == "maxlog" else "levels"
    with _device.on_device(x):
        s2 = _device.to_device(x, s2_host) if s2_host is not None else inv_s2
        sd = _device.wrap(s2, "inv_s2")
        _device.check(sd, "inv_s2", np.float32, (F,))
        tables = device_tables(constellation, kind, x)
        half = len(tables) // 2
        re, im = _axis_struct(tables[:half], kind), _axis_struct(tables[half:], kind)
        stream = _device.stream_of(x)
        lib = _lib.lib()
        if kind == "maxlog":
            st = lib.ck_llr_separable_maxlog_frames(x.ptr, F * S, S, sd.ptr, ctypes.byref(re),
                                                    ctypes.byref(im), od.ptr, stream)  # fmt: skip
        else:
            st = lib.ck_llr_separable_frames(x.ptr, F * S, S, sd.ptr, ctypes.byref(re),
                                             ctypes.byref(im), 1 if method == "exact" else 0,
                                             od.ptr, stream)  # fmt: skip
        _lib.check(st, "compute_llr_frames()")
    return out
