"""CPU oracle of the coded-modulation receiver back end.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this package, and only to check
(or time) the CUDA path.  The product package ``commkit_gb300`` never imports,
links or calls anything here.

Two layers:

* ``libck_oracle.so`` (``ck_oracle.c``), a plain-C restatement of the
  reference's CPU loops in IEEE float32: the layered min-sum / sum-product
  decoder (``commkit/coding/_numba_loops.py:37-147``) and the separable LLR
  demappers (``commkit/mapping/_numba_llr.py:35-235``), parallel over
  codewords and symbols with OpenMP.
* Pure-Python restatements of the host-side tables those loops read: the
  first-fit layer schedule (``commkit/coding/ldpc.py:283-296,422-442``), the
  quasi-cyclic lifting (``ldpc.py:183-214``), the Gray square-QAM axes
  (``commkit/mapping/gray.py:266-338``, ``_lattice.py:100-124``) and the
  opposite-level tables of the closed-form max-log
  (``commkit/mapping/_demap.py:82-106``).

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against fixtures in ``tests/golden/`` that ``tests/golden/make_golden.py``
generated by running the reference itself (its Numba kernels interpreted,
as its own CI runs them with ``NUMBA_DISABLE_JIT=1``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_SRC = _HERE / "ck_oracle.c"
_LIB_DIR = _HERE / "_build"
_LIB = _LIB_DIR / "libck_oracle.so"

_lib: ctypes.CDLL | None = None


def build(force: bool = False) -> Path:
    """Compile ``ck_oracle.c`` into ``oracle/_build/libck_oracle.so``.

    Same recipe as ``oracle/Makefile``: IEEE float32 (no contraction, no
    fast-math) so each operation rounds once, as the interpreted reference does.
    """
    if _LIB.exists() and not force and _LIB.stat().st_mtime >= _SRC.stat().st_mtime:
        return _LIB
    _LIB_DIR.mkdir(exist_ok=True)
    tmp = _LIB.with_suffix(f".{os.getpid()}.tmp")
    cmd = [
        os.environ.get("CC", "gcc"), "-O2", "-fopenmp", "-ffp-contract=off",
        "-fno-fast-math", "-fPIC", "-shared", "-std=c11", "-o", str(tmp), str(_SRC), "-lm",
    ]  # fmt: skip
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB)
    return _LIB


def lib() -> ctypes.CDLL:
    """The oracle library, built on first use."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        p = ctypes.c_void_p
        i32, i64, f32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float
        _lib.oracle_ldpc_layered.argtypes = [
            p, i64, i32, p, p, i32, i32, f32, f32, i32, i32, p, p, ctypes.c_int,
        ]  # fmt: skip
        _lib.oracle_llr_sep_maxlog.argtypes = [
            p, i64, i64, p, p, p, p, p, p, i32, i32, p, p, p, p, p, i32, i32, p, ctypes.c_int,
        ]  # fmt: skip
        _lib.oracle_llr_separable.argtypes = [
            p, i64, i64, p, p, p, p, p, i32, i32, p, p, p, p, i32, i32, i32, p, ctypes.c_int,
        ]  # fmt: skip
        _lib.oracle_llr_points.argtypes = [p, i64, i64, p, p, p, p, i32, i32, i32, p, ctypes.c_int]
        _lib.oracle_max_threads.restype = ctypes.c_int
    return _lib


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# -----------------------------------------------------------------------------
# LDPC
# -----------------------------------------------------------------------------


def first_fit(ptr: np.ndarray, variables: np.ndarray, n: int) -> np.ndarray:
    """Layer of each row (``commkit/coding/ldpc.py:422-442``).

    Rows in natural order; a row takes the lowest layer none of whose rows
    shares one of its bits.  Each bit keeps the set of layers using it as an
    integer bit mask.
    """
    masks = [0] * n
    cols = variables.tolist()
    bounds = ptr.tolist()
    color = np.empty(len(bounds) - 1, dtype=np.int64)
    for r in range(len(bounds) - 1):
        row = cols[bounds[r] : bounds[r + 1]]
        used = 0
        for v in row:
            used |= masks[v]
        free = ~used & (used + 1)  # lowest clear bit
        c = free.bit_length() - 1
        for v in row:
            masks[v] |= free
        color[r] = c
    return color


def schedule(checks: np.ndarray, variables: np.ndarray, m: int, n: int):
    """``(row_ptr, cols, layer_ptr)`` (``commkit/coding/ldpc.py:283-296``).

    ``checks``/``variables`` are the edges sorted by (row, column).  Rows
    are stably sorted by layer, so a layer's rows stay in ascending order.
    """
    ptr = np.concatenate([[0], np.cumsum(np.bincount(checks, minlength=m))])
    color = first_fit(ptr, variables, n)
    order = np.argsort(color, kind="stable")
    degree = np.diff(ptr)[order]
    row_ptr = np.concatenate([[0], np.cumsum(degree)]).astype(np.int32)
    cols = np.concatenate([variables[ptr[r] : ptr[r + 1]] for r in order]).astype(np.int32)
    layer_ptr = np.concatenate([[0], np.cumsum(np.bincount(color))]).astype(np.int32)
    return row_ptr, cols, layer_ptr


def lift(base: np.ndarray, z: int):
    """Edges of the quasi-cyclic code of ``base`` (``ldpc.py:183-214``).

    Entry ``s >= 0`` at ``(i, j)`` puts the ``z x z`` identity shifted right
    by ``s``: row ``i z + r`` has its one at column ``j z + (r + s) mod z``.
    Returns ``(checks, variables)`` sorted by (row, column), int32.
    """
    bi, bj = np.nonzero(base >= 0)
    r = np.arange(z)
    rows = (bi[:, None] * z + r).ravel()
    cols = (bj[:, None] * z + (r + base[bi, bj][:, None]) % z).ravel()
    order = np.lexsort((cols, rows))
    return rows[order].astype(np.int32), cols[order].astype(np.int32)


def ldpc_layered(app, row_ptr, cols, *, scale=0.875, offset=0.0, max_iterations=50,
                 early_stop=True, sum_product=False, threads=0):  # fmt: skip
    """Decode ``app`` ``(B, N)`` float32 in place; returns ``(iters, valid)``.

    ``commkit/coding/_numba_loops.py:109-147`` over the schedule's CSR.
    """
    app = np.ascontiguousarray(app, dtype=np.float32)
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    B, N = app.shape
    iters = np.zeros(B, np.int32)
    valid = np.zeros(B, np.uint8)
    rc = lib().oracle_ldpc_layered(
        _ptr(app), B, N, _ptr(row_ptr), _ptr(cols), row_ptr.size - 1,
        1 if sum_product else 0, np.float32(scale), np.float32(offset),
        int(max_iterations), 1 if early_stop else 0, _ptr(iters), _ptr(valid), int(threads),
    )  # fmt: skip
    if rc:
        raise RuntimeError(f"oracle_ldpc_layered failed ({rc})")
    return app, iters, valid.astype(bool)


def decode(llrs, code_tables, *, k, **method):
    """The reference's ``decode`` on a homogeneous batch: zero-padded app, then
    ``bits = app[:, :k] < 0`` (``commkit/coding/ldpc.py:539-588``).

    ``code_tables`` is ``(row_ptr, cols, N)``; ``llrs`` ``(B, n)``.
    Returns ``(bits int8 (B, k), llrs (B, n), valid, iters)``.
    """
    row_ptr, cols, n_var = code_tables
    llrs = np.asarray(llrs, dtype=np.float32)
    B, n = llrs.shape
    app = np.zeros((B, n_var), np.float32)
    app[:, :n] = llrs
    app, iters, valid = ldpc_layered(app, row_ptr, cols, **method)
    bits = (app[:, :k] < 0).astype(np.int8)
    return bits, app[:, :n].copy(), valid, iters


# -----------------------------------------------------------------------------
# LLR demapping
# -----------------------------------------------------------------------------


def gray_ask_levels(order: int) -> np.ndarray:
    """Gray ASK on ``-M+1, ..., M-1``, indexed by label (``gray.py:266-298``)."""
    k = int(np.log2(order))
    gray = np.arange(order) ^ (np.arange(order) >> 1)
    out = np.zeros(order)
    out[gray] = np.linspace(-order + 1, order - 1, order)
    return out


def gray_qam_points(order: int) -> np.ndarray:
    """Unit-power Gray square QAM indexed by label (``gray.py:301-338``):
    the high half of the label picks the in-phase level, the low half the
    quadrature one; scaled by ``sqrt(mean |p|^2)``."""
    n = int(np.log2(order)) // 2
    pam = gray_ask_levels(2**n)
    s = np.arange(order)
    pts = pam[s >> n] + 1j * pam[s & ((1 << n) - 1)]
    return pts / np.sqrt(np.mean(np.abs(pts) ** 2))


def qam_axes(order: int):
    """Separable axes of Gray square QAM (``_lattice.py:100-124``).

    Per axis ``(levels float64 ascending (L,), labels int8 (L, k_a),
    positions (k_a,))``; the in-phase axis carries the label's high bits.
    """
    k = int(np.log2(order))
    ka = k // 2
    L = 2**ka
    pts = gray_qam_points(order)
    axes = []
    for bits in (np.arange(ka), np.arange(ka, k)):
        # Level i (ascending) of either axis carries the axis label gray(i).
        vals = pts.real if bits[0] == 0 else pts.imag
        gray = np.arange(L) ^ (np.arange(L) >> 1)
        lab_of_point = (np.arange(order) >> (k - 1 - bits[-1])) & (L - 1)
        levels = np.array([vals[np.flatnonzero(lab_of_point == g)[0]] for g in gray])
        labels = ((gray[:, None] >> np.arange(ka - 1, -1, -1)) & 1).astype(np.int8)
        axes.append((levels, labels, bits.astype(np.int32)))
    return axes


def opposite_levels(labels: np.ndarray):
    """``lo``/``hi`` ``(k_a, L)`` int32 (``commkit/mapping/_demap.py:82-106``):
    per bit and level, the nearest level below / above whose bit differs,
    ``-1`` for none."""
    L, k = labels.shape
    lo = np.full((k, L), -1, np.int32)
    hi = np.full((k, L), -1, np.int32)
    for b in range(k):
        for m in range(L):
            for j in range(m - 1, -1, -1):
                if labels[j, b] != labels[m, b]:
                    lo[b, m] = j
                    break
            for j in range(m + 1, L):
                if labels[j, b] != labels[m, b]:
                    hi[b, m] = j
                    break
    return lo, hi


def packed(labels: np.ndarray) -> np.ndarray:
    """MSB-first label rows to int32 (``commkit/mapping/_demap.py:355-357``)."""
    k = labels.shape[1]
    w = 1 << np.arange(k - 1, -1, -1)
    return (labels.astype(np.int64) * w).sum(axis=1).astype(np.int32)


def inv_s2(noise_var: float) -> np.float32:
    """``float32(1 / max(nv, 1e-20))`` (``commkit/mapping/_demap.py:312``)."""
    return np.float32(1.0 / max(float(noise_var), 1e-20))


def _axis_args_maxlog(axis):
    levels, labels, pos = axis
    lev = np.ascontiguousarray(levels, dtype=np.float32)
    lab = packed(labels)
    lo, hi = opposite_levels(labels)
    return [lev, lab, lo, hi, pos.astype(np.int32)]


def llr(x, order: int, inv_s2_frames, *, method="maxlog", frame_len=None,
        closed_form=True, threads=0):  # fmt: skip
    """LLRs ``(n, k)`` float32 of complex64 symbols ``x`` ``(n,)`` on Gray
    ``order``-QAM.

    ``inv_s2_frames`` holds one float32 ``1/sigma^2`` per frame of
    ``frame_len`` symbols (one frame by default).  Max-log takes the closed
    form (``_numba_llr.py:179-235``) unless ``closed_form`` is False, then
    the level metrics (``_numba_llr.py:127-176``), as ``exact`` does.
    """
    x = np.ascontiguousarray(x, dtype=np.complex64)
    n = x.size
    s2 = np.ascontiguousarray(np.atleast_1d(inv_s2_frames), dtype=np.float32)
    frame_len = int(frame_len or max(n, 1))
    if s2.size * frame_len < n:
        raise ValueError("one inverse noise variance per frame")
    re, im = qam_axes(order)
    k = re[2].size + im[2].size
    out = np.empty((n, k), np.float32)
    xf = x.view(np.float32)
    if method == "maxlog" and closed_form:
        a_re, a_im = _axis_args_maxlog(re), _axis_args_maxlog(im)
        keep = [xf, s2, out, *a_re, *a_im]
        rc = lib().oracle_llr_sep_maxlog(
            _ptr(xf), n, frame_len, _ptr(s2), *[_ptr(a) for a in a_re],
            a_re[0].size, a_re[4].size, *[_ptr(a) for a in a_im], a_im[0].size,
            a_im[4].size, _ptr(out), int(threads),
        )  # fmt: skip
    else:
        args = []
        for levels, labels, pos in (re, im):
            lev = np.ascontiguousarray(levels, dtype=np.float32)
            logp = np.zeros(lev.size, np.float32)
            args.append([lev, logp, packed(labels), pos.astype(np.int32)])
        keep = [xf, s2, out, *args[0], *args[1]]
        rc = lib().oracle_llr_separable(
            _ptr(xf), n, frame_len, _ptr(s2), *[_ptr(a) for a in args[0]],
            args[0][0].size, args[0][3].size, *[_ptr(a) for a in args[1]],
            args[1][0].size, args[1][3].size, 1 if method == "exact" else 0,
            _ptr(out), int(threads),
        )  # fmt: skip
    del keep
    if rc:
        raise RuntimeError(f"oracle LLR failed ({rc})")
    return out


def llr_points(x, points, log_pmf, labels, k: int, inv_s2_frames, *, exact: bool = False,
               frame_len=None, threads=0):  # fmt: skip
    """LLRs ``(n, k)`` float32 of symbols ``x`` ``(n,)`` against every point
    (``commkit/mapping/_numba_llr.py:95-124``): ``points`` ``(M,)`` complex,
    ``log_pmf`` ``(M,)`` float32 and packed ``labels`` ``(M,)``; real
    symbols or points count with a zero imaginary part."""
    x = np.ascontiguousarray(x, dtype=np.complex64).reshape(-1)
    pts = np.ascontiguousarray(points, dtype=np.complex64).reshape(-1)
    logp = np.ascontiguousarray(log_pmf, dtype=np.float32)
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    n = x.size
    s2 = np.ascontiguousarray(np.atleast_1d(inv_s2_frames), dtype=np.float32)
    frame_len = int(frame_len or max(n, 1))
    if s2.size * frame_len < n:
        raise ValueError("one inverse noise variance per frame")
    out = np.empty((n, k), np.float32)
    xf, pf = x.view(np.float32), pts.view(np.float32)
    rc = lib().oracle_llr_points(_ptr(xf), n, frame_len, _ptr(s2), _ptr(pf), _ptr(logp), _ptr(lab),
                                 pts.size, int(k), 1 if exact else 0, _ptr(out), int(threads))  # fmt: skip
    if rc:
        raise RuntimeError(f"oracle_llr_points failed ({rc})")
    return out


def llr_levels(x, axes, inv_s2_frames, *, exact: bool = False, frame_len=None, threads=0):
    """LLRs ``(n, k)`` of complex64 symbols against a separable lattice given
    by its two axes, each ``(levels f32, log prior f32, packed labels i32,
    positions i32)`` (``commkit/mapping/_numba_llr.py:127-176``)."""
    x = np.ascontiguousarray(x, dtype=np.complex64).reshape(-1)
    n = x.size
    s2 = np.ascontiguousarray(np.atleast_1d(inv_s2_frames), dtype=np.float32)
    frame_len = int(frame_len or max(n, 1))
    if s2.size * frame_len < n:
        raise ValueError("one inverse noise variance per frame")
    args = [[np.ascontiguousarray(a, dtype=dt) for a, dt in zip(ax, (np.float32, np.float32, np.int32, np.int32))]
            for ax in axes]  # fmt: skip
    k = args[0][3].size + args[1][3].size
    out = np.empty((n, k), np.float32)
    xf = x.view(np.float32)
    rc = lib().oracle_llr_separable(
        _ptr(xf), n, frame_len, _ptr(s2), *[_ptr(a) for a in args[0]], args[0][0].size,
        args[0][3].size, *[_ptr(a) for a in args[1]], args[1][0].size, args[1][3].size,
        1 if exact else 0, _ptr(out), int(threads),
    )  # fmt: skip
    if rc:
        raise RuntimeError(f"oracle_llr_separable failed ({rc})")
    return out
