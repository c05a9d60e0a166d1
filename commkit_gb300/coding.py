"""LDPC codes and layered min-sum decoding: :class:`LDPCCode`, :class:`MinSum`, :func:`decode`.

Mirrors the LDPC part of ``commkit.coding``: ``LDPCCode``
(``commkit/coding/ldpc.py:53-300``; edges sorted by (row, column), the
first-fit layer schedule), ``MinSum`` (``ldpc.py:317-348``), ``decode``
(``commkit/coding/base.py:317-379``) and ``DecodeResult``
(``base.py:46-106``).  Decoding runs on the sm_103a decoder of
``csrc/ck_ldpc.cu`` behind a per-code, per-device plan; its results
(a-posteriori LLRs, hard decisions, iteration counts, syndrome flags) are
bit-identical to the reference's.  The device follows the data; host input
raises ``TypeError``.
"""

from __future__ import annotations

import ctypes
import logging
import warnings
from dataclasses import dataclass
from functools import cached_property
from typing import Any

import numpy as np

from . import _device, _lib
from .mapping import PrecisionWarning

_log = logging.getLogger(__name__)

__all__ = ["DecodeResult", "LDPCCode", "MinSum", "SumProduct", "decode", "decode_mixed", "encode"]

_HARD_LLR = 1.0


@dataclass(frozen=True)
class MinSum:
    """Layered normalized / offset min-sum (``commkit/coding/ldpc.py:317-348``):
    the check-to-bit message is ``sign * max(scale * min - offset, 0)``."""

    scale: float = 0.875
    offset: float = 0.0
    max_iterations: int = 50
    early_stop: bool = True

    def __post_init__(self) -> None:
        s = float(self.scale)
        if not np.isfinite(s) or not 0.0 < s <= 1.0:
            raise ValueError(f"scale must be in (0, 1], got {self.scale}.")
        o = float(self.offset)
        if not np.isfinite(o) or o < 0.0:
            raise ValueError(f"offset must be finite and >= 0, got {self.offset}.")
        _check_iterations(self.max_iterations)


@dataclass(frozen=True)
class SumProduct:
    """Layered sum-product (``commkit/coding/ldpc.py:351-371``)."""

    max_iterations: int = 50
    early_stop: bool = True

    def __post_init__(self) -> None:
        _check_iterations(self.max_iterations)


def _check_iterations(v: Any) -> None:
    if isinstance(v, bool) or not isinstance(v, (int, np.integer)) or v < 1:
        raise ValueError(f"max_iterations must be an integer >= 1, got {v!r}.")


@dataclass(frozen=True, eq=False)
class DecodeResult:
    """Output of :func:`decode`, arrays on the input's device (``base.py:46-106``)."""

    bits: Any
    llrs: Any | None
    valid: Any
    iterations: Any
    checked: bool


class LDPCCode:
    """LDPC code given by the edges of its sparse parity-check matrix.

    ``checks``/``variables``: row and column of each nonzero of ``H``
    (``(E,)`` integers without duplicates); ``num_checks`` m,
    ``num_variables`` N, ``punctured`` trailing parity bits not sent.
    Information bits are the first ``k = N - m`` codeword bits: the parity
    part (last m columns) must be invertible, as for the reference's
    "accumulate" and "inverse" encoders (``ldpc.py:445-481``).
    """

    def __init__(self, checks: Any, variables: Any, num_checks: int, num_variables: int,
                 punctured: int = 0):  # fmt: skip
        rows = np.asarray(checks)
        cols = np.asarray(variables)
        m, n = int(num_checks), int(num_variables)
        if rows.ndim != 1 or rows.shape != cols.shape or rows.size == 0:
            raise ValueError("checks and variables must be equal-length 1-D arrays.")
        if rows.dtype.kind not in "iu" or cols.dtype.kind not in "iu":
            raise TypeError(f"checks and variables must be integers, got {rows.dtype} and {cols.dtype}.")
        if m < 1 or n <= m:
            raise ValueError(f"need 1 <= num_checks < num_variables, got {m} and {n}.")
        if rows.min() < 0 or rows.max() >= m or cols.min() < 0 or cols.max() >= n:
            raise ValueError("checks or variables out of range.")
        order = np.lexsort((cols, rows))
        rows, cols = rows[order].astype(np.int32), cols[order].astype(np.int32)
        flat = rows.astype(np.int64) * n + cols
        if np.any(flat[1:] == flat[:-1]):
            raise ValueError("H has duplicate entries.")
        if np.bincount(rows, minlength=m).min() < 2:
            raise ValueError("every parity check needs at least two bits.")
        p = int(punctured)
        if p < 0:
            raise ValueError(f"punctured must be >= 0, got {punctured}.")
        if p > m:
            # The information bits are the first N - m.
            raise ValueError("punctured bits must be parity bits.")
        rows.setflags(write=False)
        cols.setflags(write=False)
        self.checks, self.variables = rows, cols
        self.num_checks, self.num_variables, self.punctured = m, n, p
        self._plans: dict[int, _Plan] = {}
        # Per device, what the per-call extension needs to decode this code.
        self._calls_entries: list | None = None

    @classmethod
    def quasi_cyclic(cls, base: Any, *, lifting: int, punctured: int = 0) -> LDPCCode:
        """Quasi-cyclic code of a base matrix of circulant shifts (``ldpc.py:183-214``):
        ``s >= 0`` places the identity shifted right by ``s`` (row ``r`` has its
        one at column ``(r + s) mod Z``), ``-1`` a zero block."""
        b = np.asarray(base)
        z = int(lifting)
        if z < 1:
            raise ValueError("lifting must be >= 1.")
        if b.ndim != 2 or b.size == 0 or b.dtype.kind not in "iu":
            raise ValueError("base must be a non-empty 2-D integer matrix.")
        if b.min() < -1:
            raise ValueError("base entries must be shifts >= 0 or -1.")
        # One edge per (nonzero block, row within it): block (i, j) of shift s
        # links check i z + t to variable j z + (t + s) mod z, t = 0 .. z - 1.
        blocks = np.argwhere(b >= 0)
        t = np.tile(np.arange(z), len(blocks))
        shift = np.repeat(b[blocks[:, 0], blocks[:, 1]], z)
        checks = np.repeat(blocks[:, 0] * z, z) + t
        variables = np.repeat(blocks[:, 1] * z, z) + (t + shift) % z
        code = cls(checks, variables, b.shape[0] * z, b.shape[1] * z, punctured)
        _warn_if_4_cycles(code)
        return code

    @classmethod
    def from_parity_check(cls, h: Any, *, punctured: int = 0) -> LDPCCode:
        """The code of a 0/1 parity-check matrix ``(m, N)``, dense or SciPy
        sparse (``ldpc.py:146-181``); logs a warning when two checks share
        two bits (a 4-cycle)."""
        import scipy.sparse

        if scipy.sparse.issparse(h):
            if h.ndim != 2:
                raise ValueError(f"parity_check must be 2-D, got {h.ndim}-D.")
            coo = scipy.sparse.coo_array(h)
            coo.sum_duplicates()
            coo.eliminate_zeros()
            if np.any(coo.data != 1):
                raise ValueError("parity_check must contain only 0 and 1.")
            rows, cols, shape = coo.row, coo.col, coo.shape
        else:
            h = np.asarray(h)
            if h.ndim != 2:
                raise ValueError(f"parity_check must be 2-D, got {h.ndim}-D.")
            if np.any((h != 0) & (h != 1)):
                raise ValueError("parity_check must contain only 0 and 1.")
            rows, cols = np.nonzero(h)
            shape = h.shape
        code = cls(rows, cols, shape[0], shape[1], punctured)
        _warn_if_4_cycles(code)
        return code

    @property
    def n(self) -> int:
        """Transmitted bits per codeword."""
        return self.num_variables - self.punctured

    @cached_property
    def k(self) -> int:
        """Information bits per codeword: N - rank(H) (``ldpc.py:122-125``)."""
        return int(self._info.size)

    @cached_property
    def _info(self) -> np.ndarray:
        """The information columns, increasing (``commkit/coding/ldpc.py:445-481``):
        the first N - m when the parity part (the last m columns) is
        invertible, else the columns that are not pivots of H's reduced row
        echelon form with pivots taken from the last column backwards."""
        m, n = self.num_checks, self.num_variables
        if _parity_invertible(self):
            info = np.arange(n - m, dtype=np.int64)
        else:
            info = _generator(self)[0].astype(np.int64)
        info.setflags(write=False)
        return info

    @property
    def _leading_info(self) -> bool:
        """True when the information columns are the first k (remembered)."""
        lead = self.__dict__.get("_leading_memo")
        if lead is None:
            lead = self.__dict__["_leading_memo"] = self.k == 0 or int(self._info[-1]) == self.k - 1
        return lead

    @property
    def rate(self) -> float:
        return float(self.k / self.n)

    def __repr__(self) -> str:
        return f"LDPCCode(n={self.n}, k={self.k})"

    @cached_property
    def _schedule(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """``(row_ptr, cols, layer_ptr)``: CSR of H with rows in first-fit
        layer order (``ldpc.py:283-296``), computed natively
        (``ck_ldpc_schedule``)."""
        m, n, E = self.num_checks, self.num_variables, self.checks.size
        row_ptr = np.empty(m + 1, np.int32)
        cols = np.empty(E, np.int32)
        layer_ptr = np.empty(m + 1, np.int32)
        num = ctypes.c_int32(0)
        st = _lib.lib().ck_ldpc_schedule(
            self.checks.ctypes.data, self.variables.ctypes.data, E, m, n, row_ptr.ctypes.data,
            cols.ctypes.data, layer_ptr.ctypes.data, ctypes.byref(num),
        )  # fmt: skip
        _lib.check(st, "LDPCCode schedule")
        out = (row_ptr, cols, layer_ptr[: num.value + 1].copy())
        for a in out:
            a.setflags(write=False)
        return out

    @cached_property
    def _encoder(self) -> _Encoder:
        """How the code encodes on the device (``commkit/coding/ldpc.py:445-486``)."""
        return _build_encoder(self)

    def _plan(self, device: int) -> _Plan:
        plan = self._plans.get(device)
        if plan is None:
            plan = self._plans[device] = _Plan(*self._schedule, self.num_checks, self.num_variables)
            from .tuning import apply_cached

            apply_cached(self, plan, device)
        return plan


# Largest parity part encoded through a dense inverse, and largest H reduced
# to a systematic generator (the reference's _MAX_INVERSE and _MAX_DENSE,
# commkit/coding/ldpc.py:46-48).
_MAX_INVERSE = 8192
_MAX_DENSE = 1 << 27


@dataclass(frozen=True)
class _Encoder:
    """Information columns of H as CSR (``info_row_ptr``, ``info_cols``) and
    the parity part: an accumulator of ``stride`` (``p_j = s_j + p_{j-stride}``)
    or the packed rows of ``H_p^-1`` (``inverse``, ``(m, ceil(m/32))`` uint32);
    or, for a parity part that is not invertible, ``generator`` =
    ``(info columns, pivot columns, packed generator rows)`` of
    :func:`_generator`, with the CSR empty and ``stride`` 0."""

    info_row_ptr: np.ndarray
    info_cols: np.ndarray
    stride: int
    inverse: np.ndarray | None
    generator: tuple | None = None

    def scratch_bytes(self, R: int, m: int, k: int) -> int:
        """Device scratch that encoding ``R`` frames takes."""
        if self.generator is not None:
            return 4 * R * ((k + 31) // 32)
        return R * m + (4 * R * ((m + 31) // 32) + 4 if self.inverse is not None else 0)


def _build_encoder(code: LDPCCode) -> _Encoder:
    """``s = H_info u``, then the parity part by the cheapest exact rule: an
    accumulator when every parity column c has the rows c and c + g (the
    last g only c) -- g = 1 is the reference's "accumulate" kind, g = Z a
    block dual-diagonal of identities -- else a GF(2) inverse of ``H_p`` (the
    reference's "inverse" kind, ``commkit/coding/ldpc.py:445-475``)."""
    m, n = code.num_checks, code.num_variables
    k = n - m
    rows, cols = code.checks.astype(np.int64), code.variables.astype(np.int64)
    par = cols >= k
    ir, ic = rows[~par], cols[~par]
    order = np.lexsort((ic, ir))
    row_ptr = np.concatenate([[0], np.cumsum(np.bincount(ir, minlength=m))]).astype(np.int32)
    info_cols = ic[order].astype(np.int32)
    pr, pc = rows[par], cols[par] - k
    got = np.sort(pr * m + pc)
    second = np.sort(pr[(pc == 0) & (pr > 0)])
    g = int(second[0]) if second.size else max(1, m)
    c = np.arange(m)
    want = np.sort(np.concatenate([c * m + c, (c[c + g < m] + g) * m + c[c + g < m]]))
    if got.size == want.size and np.array_equal(got, want):
        return _Encoder(row_ptr, info_cols, g, None)
    if m <= _MAX_INVERSE and _parity_invertible(code):
        return _Encoder(row_ptr, info_cols, 0, _gf2_inverse_packed(pr, pc, m))
    empty = np.zeros(1, np.int32)
    return _Encoder(empty, empty[:0], 0, None, _generator(code))


def _gf2_inverse_packed(pr: np.ndarray, pc: np.ndarray, m: int) -> np.ndarray:
    """Rows of the inverse of the m x m GF(2) matrix with ones at (pr, pc),
    packed 32 columns to a uint32 (column j at bit j % 32 of word j // 32),
    by Gauss-Jordan elimination on [H_p | I] in 64-bit words."""
    w = (m + 63) // 64
    aug = np.zeros((m, 2 * w), np.uint64)
    one = np.uint64(1)
    np.bitwise_or.at(aug, (pr, pc // 64), np.left_shift(one, (pc % 64).astype(np.uint64)))
    idx = np.arange(m)
    np.bitwise_or.at(aug, (idx, w + idx // 64), np.left_shift(one, (idx % 64).astype(np.uint64)))
    for col in range(m):
        word, bit = col // 64, one << np.uint64(col % 64)
        hits = np.flatnonzero(aug[col:, word] & bit)
        if hits.size == 0:
            raise NotImplementedError("the parity part of H is singular; such codes are not supported")
        piv = col + hits[0]
        if piv != col:
            aug[[col, piv]] = aug[[piv, col]]
        others = np.flatnonzero(aug[:, word] & bit)
        others = others[others != col]
        aug[others] ^= aug[col]
    inv64 = np.ascontiguousarray(aug[:, w:])
    inv32 = inv64.view(np.uint32)  # little-endian: word j // 32 holds columns j
    return np.ascontiguousarray(inv32[:, : (m + 31) // 32])


def _parity_invertible(code: LDPCCode) -> bool:
    """Whether the parity part ``H_p`` (last m columns) is invertible over GF(2).

    Lower triangular with a unit diagonal (dual-diagonal / accumulate parts)
    is settled from the edges; otherwise by elimination on packed bits, for
    m up to 16384 (a larger H is beyond the generator's size limit as well,
    so the answer "no" then ends in :func:`_generator`'s ``ValueError``).
    """
    m, n = code.num_checks, code.num_variables
    k = n - m
    rows, cols = code.checks, code.variables
    par = cols >= k
    pr, pc = rows[par].astype(np.int64), cols[par].astype(np.int64) - k
    diag = np.zeros(m, bool)
    diag[pr[pr == pc]] = True
    if diag.all() and not np.any(pc > pr):
        return True
    if m > 16384:
        return False
    words = (m + 63) // 64
    mat = np.zeros((m, words), np.uint64)
    np.bitwise_or.at(mat, (pr, pc // 64), np.left_shift(np.uint64(1), (pc % 64).astype(np.uint64)))
    r = 0
    for c in range(m):
        w, bit = c // 64, np.uint64(1) << np.uint64(c % 64)
        hits = np.flatnonzero(mat[r:, w] & bit)
        if hits.size == 0:
            return False
        piv = r + hits[0]
        if piv != r:
            mat[[r, piv]] = mat[[piv, r]]
        below = r + 1 + np.flatnonzero(mat[r + 1 :, w] & bit)
        mat[below] ^= mat[r]
        r += 1
    return True


def _generator(code: LDPCCode) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """``(info, pivots, gen)`` of H's reduced row echelon form over GF(2),
    pivot columns chosen from the last column backwards (the reference's
    ``row_reduce(h, reverse=True)``, ``commkit/coding/_gf2.py:45-88``, as its
    "dense" encoder uses it, ``commkit/coding/ldpc.py:476-481``).

    ``pivots`` (rank,) int32 is the pivot column of each reduced row and
    ``info`` (N - rank,) int32 the other columns, increasing; codeword bit
    ``pivots[i]`` is the GF(2) sum of the information bits where reduced row
    i has a one.  ``gen`` packs those rows over the information columns,
    ``(rank, ceil(k/32))`` uint32 (information bit j at bit j % 32 of word
    j // 32).  Column j is a pivot exactly when it is independent of the
    columns to its right, so the split does not depend on how the
    elimination is carried out.  Cached on the code.
    """
    got = code.__dict__.get("_generator_tables")
    if got is not None:
        return got
    m, n = code.num_checks, code.num_variables
    if m * n > _MAX_DENSE:
        raise ValueError(
            f"LDPCCode ({m} x {n}): the parity part is neither dual-diagonal nor "
            "invertible, and H is too large for a dense systematic generator."
        )
    words = (n + 63) // 64
    one = np.uint64(1)
    h = np.zeros((m, words), np.uint64)
    cols = code.variables.astype(np.int64)
    np.bitwise_or.at(h, (code.checks.astype(np.int64), cols // 64), np.left_shift(one, (cols % 64).astype(np.uint64)))
    pivots: list[int] = []
    r = 0
    for col in range(n - 1, -1, -1):
        if r == m:
            break
        w, bit = col // 64, one << np.uint64(col % 64)
        hits = np.flatnonzero(h[r:, w] & bit)
        if hits.size == 0:
            continue
        piv = r + int(hits[0])
        if piv != r:
            h[[r, piv]] = h[[piv, r]]
        others = np.flatnonzero(h[:, w] & bit)
        h[others[others != r]] ^= h[r]
        pivots.append(col)
        r += 1
    piv = np.asarray(pivots, np.int32)
    info = np.setdiff1d(np.arange(n, dtype=np.int32), piv)
    dense = np.unpackbits(h[:r].view(np.uint8), axis=1, bitorder="little")[:, :n]
    k = info.size
    sel = np.zeros((r, (k + 31) // 32 * 32), np.uint8)
    sel[:, :k] = dense[:, info]
    gen = np.packbits(sel, axis=1, bitorder="little").view(np.uint32)
    for a in (info, piv, gen):
        a.setflags(write=False)
    out = (info, piv, np.ascontiguousarray(gen))
    code.__dict__["_generator_tables"] = out
    return out


class _Plan:
    """A ``ck_ldpc_plan`` on one device, destroyed with the object."""

    def __init__(self, row_ptr, cols, layer_ptr, m: int, n: int):
        handle = ctypes.c_void_p()
        st = _lib.lib().ck_ldpc_plan_create(
            row_ptr.ctypes.data, cols.ctypes.data, layer_ptr.ctypes.data, m, n,
            layer_ptr.size - 1, ctypes.byref(handle),
        )  # fmt: skip
        _lib.check(st, "LDPC plan")
        self.handle = handle
        info = _lib.PlanInfo()
        _lib.check(_lib.lib().ck_ldpc_plan_get_info(handle, ctypes.byref(info)), "plan info")
        self.info = {name: getattr(info, name) for name, _ in _lib.PlanInfo._fields_}

    def set_launch(self, threads_per_frame: int = 0, frames_per_block: int = 0,
                   placement: int = 0) -> None:  # fmt: skip
        cfg = _lib.Launch(threads_per_frame, frames_per_block, placement)
        _lib.check(_lib.lib().ck_ldpc_plan_set_launch(self.handle, ctypes.byref(cfg)), "set_launch")
        self.__dict__.pop("_ws_need", None)  # workspace sizes depend on the launch shape

    def get_launch(self) -> tuple[int, int, int]:
        cfg = _lib.Launch()
        _lib.check(_lib.lib().ck_ldpc_plan_get_launch(self.handle, ctypes.byref(cfg)), "get_launch")
        return cfg.threads_per_frame, cfg.frames_per_block, cfg.placement

    def resolved_launch(self, rule: int = _lib.CK_LDPC_MIN_SUM) -> tuple[int, int, int]:
        """(threads per frame, frames per block, placement) a decode by
        ``rule`` runs with now: the setting resolved on the plan's device
        (current), the placement the one actually used."""
        cfg = _lib.Launch()
        st = _lib.lib().ck_ldpc_plan_resolved_launch(self.handle, int(rule), ctypes.byref(cfg))
        _lib.check(st, "resolved_launch")
        return cfg.threads_per_frame, cfg.frames_per_block, cfg.placement

    def set_specialise(self, mode: int) -> None:
        """``_lib.CK_LDPC_SPECIALISE_{AUTO,OFF,ON}``: whether min-sum decodes
        of this circulant code run its code-specialised kernel."""
        _lib.check(_lib.lib().ck_ldpc_plan_set_specialise(self.handle, int(mode)), "set_specialise")

    def specialisation(self) -> tuple[int, int, str]:
        """(mode, state, reason): state 1 compiled, 0 not yet, -1 unavailable
        (reason says why)."""
        mode, state = ctypes.c_int32(), ctypes.c_int32()
        lib = _lib.lib()
        _lib.check(lib.ck_ldpc_plan_get_specialise(self.handle, ctypes.byref(mode), ctypes.byref(state)),
                   "get_specialise")  # fmt: skip
        return mode.value, state.value, (_lib.last_error() if state.value < 0 else "")

    def stream_workspace(self, like: _device.DeviceArray, stream: int, rows: int, rule: int):
        """A decode workspace for ``rows`` frames kept per (stream, rule) and
        reused by later calls on that stream (grown when a call needs more),
        so a decode allocates nothing but its outputs; and the lock that
        serialises its use by host threads (a decode resets the workspace's
        frame counter and launches on the stream, and two threads
        interleaving those on one workspace would corrupt both).  Work on
        one stream runs in order, so calls never overlap on the device."""
        import threading

        cache = self.__dict__.setdefault("_stream_ws", {})
        key = (stream, rule)
        entry = cache.get(key)
        size_key = (rows, rule)
        need = self.__dict__.setdefault("_ws_need", {}).get(size_key)
        if need is None:
            need = self._ws_need[size_key] = self.workspace_size(rows, rule)
        if entry is None or entry[0].numel() < need:
            lock = entry[1] if entry is not None else threading.Lock()
            entry = cache[key] = (_device.empty(like, (max(need, 256),), np.uint8), lock)
        return entry

    def workspace_size(self, frames: int, rule: int = _lib.CK_LDPC_MIN_SUM) -> int:
        size = ctypes.c_size_t(0)
        st = _lib.lib().ck_ldpc_workspace_size(self.handle, int(frames), int(rule), ctypes.byref(size))
        _lib.check(st, "workspace size")
        return int(size.value)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib.lib().ck_ldpc_plan_destroy(h)
            self.handle = None


def _resolve_method(method: Any) -> MinSum | SumProduct:
    if method is None:
        return _DEFAULT_METHOD
    if not isinstance(method, (MinSum, SumProduct)):
        raise TypeError(
            f"decode(): method {type(method).__name__} does not decode LDPCCode; use MinSum or SumProduct."
        )
    return method


def _rule_args(method: MinSum | SumProduct) -> tuple[int, float, float]:
    """(rule, scale, offset) of the C ABI; sum-product has neither parameter
    (``commkit/coding/ldpc.py:547-549`` passes 1 and 0).  The parameters are
    rounded to float32 and kept as Python floats, which the C call takes as
    the same float32 values (ctypes converts a NumPy scalar several
    microseconds slower); remembered on the (frozen) method object."""
    args = method.__dict__.get("_c_args")
    if args is None:
        if isinstance(method, SumProduct):
            args = (_lib.CK_LDPC_SUM_PRODUCT, 1.0, 0.0)
        else:
            args = (_lib.CK_LDPC_MIN_SUM, float(np.float32(method.scale)), float(np.float32(method.offset)))
        method.__dict__["_c_args"] = args
        # The whole call as the per-call extension takes it.
        method.__dict__["_c_call"] = args + (int(method.max_iterations), 1 if method.early_stop else 0)
    return args


_DEFAULT_METHOD = MinSum()
_METHODS = (MinSum, SumProduct)
_calls_decode = None  # the per-call extension's decode, once a code has registered


def _register_calls(code: LDPCCode, device: int, plan: _Plan) -> None:
    """Lets later ``decode`` calls of ``code`` on ``device`` (contiguous
    float32 torch LLRs, no workspace given) go straight to the per-call
    extension: the entry is the plan's handle and the code's sizes, kept in
    a list indexed by device."""
    global _calls_decode
    mod = _lib.calls()
    if mod is None:
        return
    entries = code._calls_entries
    if entries is None or len(entries) <= device:
        entries = list(entries or ()) + [None] * (device + 1 - len(entries or ()))
    entries[device] = (plan.handle.value, code.n, code.k)
    code._calls_entries = entries
    _calls_decode = mod.decode


def _as_llrs(llrs: Any, x: _device.DeviceArray):
    """float32 LLRs; integer or bool input read as hard decisions (``base.py:232-245``)."""
    import torch

    if x.kind != "torch":
        import cupy

        a = llrs
        if x.dtype.kind == "c":
            raise TypeError(f"decode(): llrs must be real, got {x.dtype}.")
        if x.dtype.kind in "biu":
            return (1.0 - 2.0 * _HARD_LLR * (a != 0)).astype(cupy.float32)
        if x.dtype == np.float64:
            warnings.warn("decode(): float64 llrs computed in float32", PrecisionWarning, stacklevel=3)
        return cupy.ascontiguousarray(a.astype(cupy.float32, copy=False))
    t = llrs
    if t.is_complex():
        raise TypeError(f"decode(): llrs must be real, got {x.dtype}.")
    if x.dtype.kind in "biu":
        return _HARD_LLR - 2.0 * _HARD_LLR * (t != 0).to(torch.float32)
    if t.dtype == torch.float64:
        warnings.warn("decode(): float64 llrs computed in float32", PrecisionWarning, stacklevel=3)
    return t.to(torch.float32).contiguous()


def decode(llrs: Any, *, code: LDPCCode, method: MinSum | SumProduct | None = None,
           workspace: Any = None) -> DecodeResult:  # fmt: skip
    """Decode LLRs of a code's transmitted bits (``commkit/coding/base.py:317-379``).

    ``llrs`` ``(N,)`` or ``(C, N)`` on a CUDA device, ``N`` a multiple of
    ``code.n``; positive means bit 0.  Returns bits int8 ``(..., B k)``,
    a-posteriori llrs float32 ``(..., B n)``, valid bool ``(..., B)`` and
    iterations int32 ``(..., B)``, all on the input's device.
    ``workspace``: optional device scratch (uint8) reused across calls, at
    least ``code._plan(dev).workspace_size(B, rule)`` bytes.
    """
    if not isinstance(code, LDPCCode):
        raise TypeError(f"decode(): code must be an LDPCCode, got {type(code).__name__}.")
    entries = code._calls_entries
    if entries is not None and workspace is None:
        # A form an earlier call registered: the extension takes it whole, or
        # returns None and the general path below runs.
        m = _DEFAULT_METHOD if method is None else method
        call = m.__dict__.get("_c_call") if isinstance(m, _METHODS) else None
        if call is not None:
            r = _calls_decode(llrs, entries, call)
            if r is not None:
                if r.__class__ is int:
                    _lib.check(r, "decode()")
                return r
    method = _resolve_method(method)
    x0 = _device.wrap(llrs, "llrs")
    if workspace is None and x0.kind == "torch" and x0.dtype == np.float32 and x0.contiguous and code._leading_info:
        return _decode_torch(llrs, x0, code, method)
    x = _as_llrs(llrs, x0)
    was_1d = x0.ndim == 1
    x2 = x.reshape(1, -1) if was_1d else x
    if x2.ndim != 2:
        raise ValueError(f"decode(): llrs must be 1-D or 2-D, got {x2.ndim}-D.")
    if x2.shape[-1] % code.n:
        raise ValueError(
            f"decode(): the last axis of llrs ({x2.shape[-1]}) must be a multiple of the block "
            f"length {code.n}."
        )
    C = x2.shape[0]
    nb = x2.shape[-1] // code.n
    rows = C * nb
    blocks = x2.reshape(rows, code.n)
    xd = _device.wrap(blocks, "llrs")
    k = code.k
    leading = code._leading_info
    if not leading and int(code._info[-1]) >= code.n:
        raise NotImplementedError(
            f"decode(): {code!r} has information columns among its punctured bits, which the "
            "a-posteriori LLRs do not hold"
        )  # fmt: skip
    out_llrs = _device.empty(xd, (rows, code.n), np.float32)
    bits = _device.empty(xd, (rows, k), np.int8)
    iters = _device.empty(xd, (rows,), np.int32)
    valid_u8 = _device.empty(xd, (rows,), np.uint8)
    if rows:
        ptr = (lambda a: a.data_ptr()) if xd.kind == "torch" else (lambda a: _device.wrap(a).ptr)
        with _device.on_device(xd):
            plan = code._plan(xd.device)
            stream = _device.stream_of(xd)
            rule, scale, offset = _rule_args(method)
            lock = None
            if workspace is None:
                workspace, lock = plan.stream_workspace(xd, stream, rows, rule)
            wsd = _device.wrap(workspace, "workspace")
            args = (plan.handle, xd.ptr, ptr(out_llrs), rows, code.n, rule, scale, offset,
                    int(method.max_iterations), 1 if method.early_stop else 0, ptr(iters), ptr(valid_u8),
                    ptr(bits) if leading else None, k if leading else 0, wsd.ptr, wsd.size, stream)  # fmt: skip
            if lock is None:
                st = _lib.lib().ck_ldpc_decode(*args)
            else:
                with lock:  # the workspace's counter reset and launch, enqueued as a pair
                    st = _lib.lib().ck_ldpc_decode(*args)
            _lib.check(st, "decode()")
            if not leading:
                # Hard decisions at the information columns (ldpc.py:582-586).
                st = _lib.lib().ck_ldpc_column_signs(
                    ptr(out_llrs), rows, code.n, _device.wrap(_info_columns(code, xd)).ptr, k, ptr(bits), stream,
                )  # fmt: skip
                _lib.check(st, "decode() bits")
    valid = valid_u8.view(_bool_dtype(xd))

    def shaped(a, size):
        a = a.reshape(C, nb * size)
        return a.reshape(-1) if was_1d else a

    return DecodeResult(bits=shaped(bits, k), llrs=shaped(out_llrs, code.n),
                        valid=shaped(valid, 1), iterations=shaped(iters, 1), checked=True)  # fmt: skip


def _decode_torch(llrs: Any, x0: _device.DeviceArray, code: LDPCCode, method: MinSum | SumProduct) -> DecodeResult:
    """``decode`` of contiguous float32 torch LLRs of a code whose information
    bits lead its codeword, with the plan's per-stream workspace: the outputs
    are allocated in their final shapes and every pointer comes straight from
    the tensors, so the host work is little more than the four allocations
    and the launch (the same kernel and results as the general path)."""
    import torch

    shape = x0.shape
    if len(shape) not in (1, 2):
        raise ValueError(f"decode(): llrs must be 1-D or 2-D, got {len(shape)}-D.")
    n, k = code.n, code.k
    last = shape[-1]
    if last % n:
        raise ValueError(
            f"decode(): the last axis of llrs ({last}) must be a multiple of the block length {n}."
        )  # fmt: skip
    nb = last // n
    C = 1 if len(shape) == 1 else shape[0]
    rows = C * nb
    dev = llrs.device
    lead = () if len(shape) == 1 else (C,)
    out_llrs = torch.empty(lead + (nb * n,), dtype=torch.float32, device=dev)
    bits = torch.empty(lead + (nb * k,), dtype=torch.int8, device=dev)
    iters = torch.empty(lead + (nb,), dtype=torch.int32, device=dev)
    valid = torch.empty(lead + (nb,), dtype=torch.bool, device=dev)
    if rows:
        with _device.on_device(x0):
            plan = code._plan(x0.device)
            stream = _device.stream_of(x0)
            rule, scale, offset = _rule_args(method)
            ws, lock = plan.stream_workspace(x0, stream, rows, rule)
            with lock:
                st = _lib.lib().ck_ldpc_decode(
                    plan.handle, x0.ptr, out_llrs.data_ptr(), rows, n, rule, scale, offset,
                    int(method.max_iterations), 1 if method.early_stop else 0, iters.data_ptr(),
                    valid.data_ptr(), bits.data_ptr(), k, ws.data_ptr(), ws.numel(), stream,
                )  # fmt: skip
            _lib.check(st, "decode()")
            _register_calls(code, x0.device, plan)
    return DecodeResult(bits=bits, llrs=out_llrs, valid=valid, iterations=iters, checked=True)


def _warn_if_4_cycles(code: LDPCCode) -> None:
    """Logs a warning when two checks share two or more bits, a 4-cycle of
    the Tanner graph on which belief propagation degrades, as the reference
    does when it builds a code (``ldpc.py:415-419``): the off-diagonal
    entries of H H^T count the bits each pair of checks shares."""
    import scipy.sparse

    h = scipy.sparse.csr_array((np.ones(code.checks.size, np.int32), (code.checks, code.variables)),
                               shape=(code.num_checks, code.num_variables))  # fmt: skip
    shared = (h @ h.T).tocoo()
    if np.any(shared.data[shared.row != shared.col] > 1):
        _log.warning("%r has 4-cycles; belief propagation degrades on them.", code)


def _encoder_tables(code: LDPCCode, like: _device.DeviceArray) -> tuple:
    """The encoder's tables on ``like``'s device, cached per code and device."""
    per = code.__dict__.setdefault("_enc_dev", {})
    t = per.get(like.device)
    if t is None:
        e = code._encoder
        if e.generator is not None:
            info, piv, gen = e.generator
            t = (_device.to_device(like, info), _device.to_device(like, piv),
                 _device.to_device(like, gen.view(np.int32)))  # fmt: skip
        else:
            inv = None if e.inverse is None else _device.to_device(like, e.inverse.view(np.int32))
            t = (_device.to_device(like, e.info_row_ptr), _device.to_device(like, e.info_cols), inv)
        per[like.device] = t
    return t


def _info_columns(code: LDPCCode, like: _device.DeviceArray):
    """The information columns as int32 on ``like``'s device, cached."""
    per = code.__dict__.setdefault("_info_dev", {})
    t = per.get(like.device)
    if t is None:
        t = per[like.device] = _device.to_device(like, code._info.astype(np.int32))
    return t


def _require_leading_info(code: LDPCCode, what: str) -> None:
    if not code._leading_info:
        raise NotImplementedError(
            f"{what}: the information columns of {code!r} are not the first k (its parity part is not "
            "invertible); decode() and encode() take such codes"
        )  # fmt: skip


def encode_blocks(code: LDPCCode, info: Any, words: Any = None, scratch: Any = None) -> Any:
    """``(R, k)`` int8 information rows on a CUDA device to ``(R, n)`` int8
    codewords, systematic (``commkit/coding/ldpc.py:511-536``).  ``words``
    and ``scratch`` (int8, ``code._encoder.scratch_bytes(R, m, k)`` bytes)
    may be preallocated."""
    xd = _device.wrap(info, "info")
    _device.check(xd, "info", np.int8, (None, code.k))
    R = xd.shape[0]
    m, k, n = code.num_checks, code.k, code.n
    if words is None:
        words = _device.empty(xd, (R, n), np.int8)
    wd = _device.wrap(words, "words")
    _device.check(wd, "words", np.int8, (R, n))
    if R == 0:
        return words
    e = code._encoder
    if scratch is None:
        scratch = _device.empty(xd, (e.scratch_bytes(R, m, k),), np.int8)
    sd = _device.wrap(scratch, "scratch")
    with _device.on_device(xd):
        if e.generator is not None:
            info_cols, piv, gen = _encoder_tables(code, xd)
            st = _lib.lib().ck_ldpc_encode_generator(
                xd.ptr, R, k, e.generator[1].size, n, _device.wrap(info_cols).ptr, _device.wrap(piv).ptr,
                _device.wrap(gen).ptr, sd.ptr, sd.size, wd.ptr, _device.stream_of(xd),
            )  # fmt: skip
        else:
            rp, ci, inv = _encoder_tables(code, xd)
            st = _lib.lib().ck_ldpc_encode(
                xd.ptr, R, k, m, n, _device.wrap(rp).ptr, _device.wrap(ci).ptr, e.stride,
                None if inv is None else _device.wrap(inv).ptr, sd.ptr, sd.size, wd.ptr, _device.stream_of(xd),
            )  # fmt: skip
        _lib.check(st, "encode()")
    return words


def encode(bits: Any, *, code: LDPCCode) -> Any:
    """Encode information bits (``commkit/coding/base.py:248-290``).

    ``bits`` ``(N,)`` or ``(C, N)`` integers 0/1 on a CUDA device, ``N`` a
    multiple of ``code.k``; returns int8 ``(..., N / k * n)`` on the same
    device, each block ``[info | parity]`` (punctured parity bits left out),
    or, for a code whose parity part is not invertible, the information bits
    at ``code``'s information columns and the parity bits at the others.
    """
    if not isinstance(code, LDPCCode):
        raise TypeError(f"encode(): code must be an LDPCCode, got {type(code).__name__}.")
    x = _device.wrap(bits, "bits")
    if x.dtype.kind not in "biu":
        raise TypeError(f"encode(): bits must be integers or bool, got {x.dtype}.")
    t = bits
    if x.kind == "torch":
        import torch

        if x.dtype.kind != "b" and t.numel() and bool(((t < 0) | (t > 1)).any()):
            raise ValueError("encode(): bits must be 0 or 1.")
        t = t.to(torch.int8)
    else:
        if x.dtype.kind != "b" and x.size and bool(((t < 0) | (t > 1)).any()):
            raise ValueError("encode(): bits must be 0 or 1.")
        t = t.astype(np.int8)
    was_1d = x.ndim == 1
    t2 = t.reshape(1, -1) if was_1d else t
    if t2.ndim != 2:
        raise ValueError(f"encode(): bits must be 1-D or 2-D, got {t2.ndim}-D.")
    if t2.shape[-1] % code.k:
        raise ValueError(f"encode(): the last axis of bits ({t2.shape[-1]}) must be a multiple of k = {code.k}.")
    C, nb = t2.shape[0], t2.shape[-1] // code.k
    blocks = t2.reshape(C * nb, code.k)
    if x.kind == "torch":
        blocks = blocks.contiguous()
    out = encode_blocks(code, blocks).reshape(C, nb * code.n)
    return out.reshape(-1) if was_1d else out


def _bool_dtype(xd: _device.DeviceArray):
    if xd.kind == "torch":
        import torch

        return torch.bool
    return np.bool_


def decode_mixed(batches, *, workspace: Any = None, outputs: list | None = None) -> list[DecodeResult]:
    """Decode frames of several quasi-cyclic codes in one launch.

    ``batches`` is a sequence of ``(llrs, code, method)``: per code, LLRs
    ``(B, n)`` (or ``(B n,)``) float32 on one CUDA device.  One persistent
    kernel decodes them all; each block works on one code at a time and
    moves to the code with the most frames left when its queue empties
    (``ck_ldpc_decode_mixed``).  Returns one :class:`DecodeResult` per batch,
    each bit-identical to ``decode(llrs, code=code, method=method)``.
    """
    items = []
    device = None
    for llrs, code, method in batches:
        if not isinstance(code, LDPCCode):
            raise TypeError(f"decode_mixed(): code must be an LDPCCode, got {type(code).__name__}.")
        _require_leading_info(code, "decode_mixed()")
        method = _resolve_method(method)
        if not isinstance(method, MinSum):
            raise NotImplementedError("decode_mixed(): mixed launches decode with MinSum; decode "
                                      "SumProduct batches with decode()")  # fmt: skip
        x0 = _device.wrap(llrs, "llrs")
        x = _as_llrs(llrs, x0).reshape(-1)
        if x.shape[0] % code.n:
            raise ValueError(f"decode_mixed(): {x.shape[0]} LLRs is not a multiple of n = {code.n}.")
        B = x.shape[0] // code.n
        xd = _device.wrap(x, "llrs")
        if device is None:
            device = xd
        elif xd.device != device.device:
            raise ValueError("decode_mixed(): all batches must be on one device.")
        if outputs is not None:
            # Preallocated (llrs (B, n) f32, bits (B, k) i8, iters (B,) i32, valid (B,) u8):
            # nothing is allocated, so the call can be captured in a CUDA graph.
            out, bits, iters, valid = outputs[len(items)]
        else:
            out = _device.empty(xd, (B, code.n), np.float32)
            bits = _device.empty(xd, (B, code.k), np.int8)
            iters = _device.empty(xd, (B,), np.int32)
            valid = _device.empty(xd, (B,), np.uint8)
        items.append((x, xd, code, method, B, out, bits, iters, valid))
    if len(items) > 4:
        raise ValueError("decode_mixed(): at most 4 codes per launch.")
    results = []
    if items:
        with _device.on_device(device):
            arr = (_lib.Batch * len(items))()
            for i, (x, xd, code, method, B, out, bits, iters, valid) in enumerate(items):
                plan = code._plan(xd.device)
                arr[i] = _lib.Batch(plan.handle, xd.ptr, _device.wrap(out).ptr, B, code.n,
                                    *_rule_args(method), int(method.max_iterations),
                                    1 if method.early_stop else 0, _device.wrap(iters).ptr,
                                    _device.wrap(valid).ptr, _device.wrap(bits).ptr, code.k)  # fmt: skip
            lib = _lib.lib()
            if workspace is None:
                need = ctypes.c_size_t(0)
                _lib.check(lib.ck_ldpc_mixed_workspace_size(arr, len(items), ctypes.byref(need)),
                           "decode_mixed()")  # fmt: skip
                workspace = _device.empty(device, (max(int(need.value), 256),), np.uint8)
            wsd = _device.wrap(workspace, "workspace")
            st = lib.ck_ldpc_decode_mixed(arr, len(items), wsd.ptr, wsd.size, _device.stream_of(device))
            _lib.check(st, "decode_mixed()")
    for x, xd, code, method, B, out, bits, iters, valid in items:
        results.append(DecodeResult(bits=bits, llrs=out, valid=valid.view(_bool_dtype(xd)),
                                    iterations=iters, checked=True))  # fmt: skip
    return results
