"""Kernel registry with the reference's launcher interface.

``get_kernel(name, **spec)`` returns a launcher with the signature, argument
meaning and error behaviour of the reference's
(``commkit/_cuda/__init__.py:35-81``): ``TypeError`` for a wrong dtype,
``ValueError`` for a wrong shape, size or non-contiguous array, outputs
allocated by the launcher on the input's device, work queued on the
input's current stream with no synchronization.  Behind each launcher is an
sm_103a kernel of ``libck_gb300.so``:

======================  ====================================  ===========================
name                    reference launcher                    C ABI
======================  ====================================  ===========================
llr                     commkit/_cuda/llr.py:37-84            ck_llr_points
llr_separable_maxlog    commkit/_cuda/llr.py:150-206          ck_llr_separable_maxlog
llr_separable           commkit/_cuda/llr.py:87-147           ck_llr_separable
ldpc_layered            commkit/_cuda/coding.py:11-69         ck_ldpc_plan_create + ck_ldpc_decode
======================  ====================================  ===========================

:mod:`commkit_gb300.plugin` installs these factories into the reference's
own registry, so its ``compute_llr`` / ``decode`` run them unchanged.
"""

from __future__ import annotations

import ctypes
import weakref
from collections.abc import Callable
from typing import Any

import numpy as np

from . import _device, _lib

LLR_MAX_K = _lib.CK_LLR_MAX_K


def _llr_factory() -> Callable:
    """Max-log or exact LLRs from the metrics of every point."""

    def launch(x: Any, points: Any, log_pmf: Any, labels: Any, *, k: int, inv_s2: float,
               exact: bool) -> Any:  # fmt: skip
        """LLRs of the ``(n,)`` complex64 symbols ``x``, shape ``(n, k)``;
        ``points`` ``(M,)`` complex64, ``log_pmf`` ``(M,)`` float32 and
        ``labels`` ``(M,)`` int32 (each point's k-bit label, MSB first)."""
        if not 1 <= k <= LLR_MAX_K:
            raise ValueError(f"bits per symbol must be in [1, {LLR_MAX_K}], got {k}")
        xd, pd = _device.wrap(x, "x"), _device.wrap(points, "points")
        _device.check(xd, "x", np.complex64, (None,))
        _device.check(pd, "points", np.complex64, (None,))
        M = pd.shape[0]
        if M < 1:
            raise ValueError(f"points must be non-empty, got M={M}")
        lp, la = _device.wrap(log_pmf, "log_pmf"), _device.wrap(labels, "labels")
        _device.check(lp, "log_pmf", np.float32, (M,))
        _device.check(la, "labels", np.int32, (M,))
        n = xd.shape[0]
        if n >= 2**31:
            raise ValueError(f"at most 2**31 - 1 symbols per call, got {n}")
        out = _device.empty(xd, (n, k), np.float32)
        if n == 0:
            return out
        with _device.on_device(xd):
            st = _lib.lib().ck_llr_points(
                xd.ptr, n, pd.ptr, lp.ptr, la.ptr, M, int(k), float(np.float32(inv_s2)),
                1 if exact else 0, _device.wrap(out).ptr, _device.stream_of(xd),
            )  # fmt: skip
        _lib.check(st, "llr")
        return out

    return launch


def _llr_separable_maxlog_factory() -> Callable:
    """Closed-form max-log LLRs of a uniform separable lattice."""

    def launch(x: Any, re: tuple, im: tuple, *, inv_s2: float) -> Any:
        """LLRs of the ``(n,)`` complex64 symbols ``x``, shape ``(n, k)``.

        ``re`` and ``im`` are each ``(levels, labels, lo, hi, positions)``:
        float32 and int32 ``(L,)``, int32 ``(k_axis, L)`` twice, int32
        ``(k_axis,)``; ``L >= 2`` equally spaced ascending levels.
        """
        xd = _device.wrap(x, "x")
        _device.check(xd, "x", np.complex64, (None,))
        axes = []
        for name, (lev, lab, lo, hi, pos) in (("re", re), ("im", im)):
            lv, ps = _device.wrap(lev, f"{name} levels"), _device.wrap(pos, f"{name} positions")
            _device.check(lv, f"{name} levels", np.float32, (None,))
            _device.check(ps, f"{name} positions", np.int32, (None,))
            L, kb = lv.shape[0], ps.shape[0]
            if not 1 <= kb <= LLR_MAX_K:
                raise ValueError(f"bits of the {name} axis must be in [1, {LLR_MAX_K}], got {kb}")
            if L < 2:
                raise ValueError(f"the {name} axis needs at least 2 levels, got {L}")
            la = _device.wrap(lab, f"{name} labels")
            lod, hid = _device.wrap(lo, f"{name} lo"), _device.wrap(hi, f"{name} hi")
            _device.check(la, f"{name} labels", np.int32, (L,))
            _device.check(lod, f"{name} lo", np.int32, (kb, L))
            _device.check(hid, f"{name} hi", np.int32, (kb, L))
            axes.append(_lib.AxisMaxlog(lv.ptr, la.ptr, lod.ptr, hid.ptr, ps.ptr, L, kb))
        k = axes[0].k + axes[1].k
        if k > LLR_MAX_K:
            raise ValueError(f"bits per symbol must be at most {LLR_MAX_K}, got {k}")
        n = xd.shape[0]
        if n >= 2**31:
            raise ValueError(f"at most 2**31 - 1 symbols per call, got {n}")
        out = _device.empty(xd, (n, k), np.float32)
        if n == 0:
            return out
        with _device.on_device(xd):
            st = _lib.lib().ck_llr_separable_maxlog(
                xd.ptr, n, ctypes.byref(axes[0]), ctypes.byref(axes[1]),
                float(np.float32(inv_s2)), _device.wrap(out).ptr, _device.stream_of(xd),
            )  # fmt: skip
        _lib.check(st, "llr_separable_maxlog")
        return out

    return launch


def _llr_separable_factory() -> Callable:
    """Max-log or exact LLRs from the metrics of each axis's levels."""

    def launch(x: Any, re: tuple, im: tuple, *, inv_s2: float, exact: bool) -> Any:
        """LLRs of the ``(n,)`` complex64 symbols ``x``, shape ``(n, k)``.

        ``re`` and ``im`` are each ``(levels, log_prior, labels, positions)``:
        float32, float32 and int32 ``(L,)``, int32 ``(k_axis,)``.
        """
        xd = _device.wrap(x, "x")
        _device.check(xd, "x", np.complex64, (None,))
        axes = []
        for name, (lev, logp, lab, pos) in (("re", re), ("im", im)):
            lv, ps = _device.wrap(lev, f"{name} levels"), _device.wrap(pos, f"{name} positions")
            _device.check(lv, f"{name} levels", np.float32, (None,))
            _device.check(ps, f"{name} positions", np.int32, (None,))
            L, kb = lv.shape[0], ps.shape[0]
            if L < 1:
                raise ValueError(f"the {name} axis needs at least 1 level, got {L}")
            if not 1 <= kb <= LLR_MAX_K:
                raise ValueError(f"bits of the {name} axis must be in [1, {LLR_MAX_K}], got {kb}")
            lp, la = _device.wrap(logp, f"{name} log prior"), _device.wrap(lab, f"{name} labels")
            _device.check(lp, f"{name} log prior", np.float32, (L,))
            _device.check(la, f"{name} labels", np.int32, (L,))
            axes.append(_lib.AxisLevels(lv.ptr, lp.ptr, la.ptr, ps.ptr, L, kb))
        k = axes[0].k + axes[1].k
        if k > LLR_MAX_K:
            raise ValueError(f"bits per symbol must be at most {LLR_MAX_K}, got {k}")
        n = xd.shape[0]
        if n >= 2**31:
            raise ValueError(f"at most 2**31 - 1 symbols per call, got {n}")
        out = _device.empty(xd, (n, k), np.float32)
        if n == 0:
            return out
        with _device.on_device(xd):
            st = _lib.lib().ck_llr_separable(
                xd.ptr, n, ctypes.byref(axes[0]), ctypes.byref(axes[1]),
                float(np.float32(inv_s2)), 1 if exact else 0, _device.wrap(out).ptr,
                _device.stream_of(xd),
            )  # fmt: skip
        _lib.check(st, "llr_separable")
        return out

    return launch


class _PlanCache:
    """Plans keyed by the schedule's device arrays.

    The reference caches those arrays per code and device
    (``commkit/backend.py:265-287``), so the same objects come back on
    every call; the first call copies them to the host once to build the
    plan.  The key holds each array's identity, device pointer, size and
    device, and entries die with the arrays; arrays that cannot be weakly
    referenced (so an entry could outlive them and a new array reuse their
    identity) get a plan per call, uncached.
    """

    def __init__(self) -> None:
        self._plans: dict[tuple, Any] = {}

    @staticmethod
    def _key_of(a: Any) -> tuple:
        d = _device.wrap(a)
        return (id(a), d.ptr, d.size, d.device)

    def get(self, row_ptr: Any, cols: Any, layer_ptr: Any, n_var: int) -> Any:
        from .coding import _Plan

        arrays = (row_ptr, cols, layer_ptr)
        key = (*(self._key_of(a) for a in arrays), n_var)
        plan = self._plans.get(key)
        if plan is None:
            host = [_to_host(a) for a in arrays]
            plan = _Plan(*host, host[0].size - 1, n_var)
            try:
                for a in arrays:
                    weakref.ref(a)
            except TypeError:
                return plan
            self._plans[key] = plan
            for a in arrays:
                weakref.finalize(a, self._plans.pop, key, None)
        return plan


def _to_host(a: Any) -> np.ndarray:
    if hasattr(a, "get"):
        return np.ascontiguousarray(a.get(), dtype=np.int32)
    if hasattr(a, "cpu"):
        return np.ascontiguousarray(a.cpu().numpy(), dtype=np.int32)
    return np.ascontiguousarray(a, dtype=np.int32)


_PLANS = _PlanCache()


def _ldpc_layered_factory(sum_product: bool = False) -> Callable:
    """Layered LDPC decoding of ``app`` in place (the reference's ``ldpc_layered``,
    ``commkit/_cuda/coding.py:11-67``); ``sum_product`` picks the check rule as
    its template argument does (``scale``/``offset`` then unused)."""
    rule = _lib.CK_LDPC_SUM_PRODUCT if sum_product else _lib.CK_LDPC_MIN_SUM

    def launch(app: Any, row_ptr: Any, cols: Any, layer_ptr: Any, *, scale: float,
               offset: float, max_iterations: int, early_stop: bool) -> tuple[Any, Any]:  # fmt: skip
        """Decode ``app`` ``(B, N)`` float32 in place; returns ``(iters, valid)``."""
        ad = _device.wrap(app, "app")
        rp, cc, lp = (_device.wrap(a, nm) for a, nm in ((row_ptr, "row_ptr"), (cols, "cols"),
                                                        (layer_ptr, "layer_ptr")))  # fmt: skip
        _device.check(ad, "app", np.float32, (None, None))
        _device.check(rp, "row_ptr", np.int32, (None,))
        _device.check(cc, "cols", np.int32, (None,))
        _device.check(lp, "layer_ptr", np.int32, (None,))
        B, N = ad.shape
        if rp.size < 2 or lp.size < 2:
            raise ValueError(
                f"row_ptr and layer_ptr need at least 2 entries, got {rp.size} and {lp.size}"
            )
        iters = _device.zeros(ad, (B,), np.int32)
        valid = _device.zeros(ad, (B,), np.uint8)
        if B == 0:
            return iters, valid.view(_bool(ad))
        with _device.on_device(ad):
            plan = _PLANS.get(row_ptr, cols, layer_ptr, N)
            ws = _device.empty(ad, (plan.workspace_size(B, rule),), np.uint8)
            st = _lib.lib().ck_ldpc_decode(
                plan.handle, ad.ptr, ad.ptr, B, N, rule, float(np.float32(scale)),
                float(np.float32(offset)), int(max_iterations), 1 if early_stop else 0,
                _device.wrap(iters).ptr, _device.wrap(valid).ptr, None, 0,
                _device.wrap(ws).ptr, _device.wrap(ws).size, _device.stream_of(ad),
            )  # fmt: skip
        _lib.check(st, "ldpc_layered")
        return iters, valid.view(_bool(ad))

    return launch


def _bool(ad: _device.DeviceArray):
    if ad.kind == "torch":
        import torch

        return torch.bool
    return np.bool_


def get_kernel(name: str, **spec: Any) -> Callable:
    """A launcher for a registered kernel (``commkit/_cuda/__init__.py:35-66``)."""
    factory = _KERNEL_FACTORIES.get(name)
    if factory is None:
        raise KeyError(f"Unknown CUDA kernel {name!r}; registered: {sorted(_KERNEL_FACTORIES)}")
    return factory(**spec)


#: Kernel name -> launcher factory (the reference's names).
_KERNEL_FACTORIES: dict[str, Callable[..., Callable]] = {
    "llr": _llr_factory,
    "llr_separable_maxlog": _llr_separable_maxlog_factory,
    "llr_separable": _llr_separable_factory,
    "ldpc_layered": _ldpc_layered_factory,
}
