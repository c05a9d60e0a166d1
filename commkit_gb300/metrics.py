"""Information rates of LLRs on the device: :func:`gmi` and :func:`ngmi`.

``commkit/metrics/information.py:40-236`` for LLR arrays: the loss
``E[log2(1 + e^{-(1 - 2 c) L})]`` over the bits of each channel, each term
in float32 as the reference computes it (``csrc/ck_sim.cu``), summed in
float64 over chunks in a fixed order, so the result does not depend on the
launch.  ``GMI = H(X) - k loss`` (bits per symbol) and ``NGMI = 1 - loss``.
"""

from __future__ import annotations

from typing import Any

import numpy as np

from . import _device, _lib
from .mapping import Constellation

__all__ = ["gmi", "ngmi"]


def _loss(llrs: Any, reference: Any, constellation: Constellation | None, num_skip_symbols: int,
          name: str) -> tuple[Any, Constellation, bool]:  # fmt: skip
    if reference is None:
        raise ValueError(f"{name}: reference bits are required for LLR arrays.")
    if constellation is None:
        raise ValueError(f"{name}: constellation is required for LLR arrays.")
    x = _device.wrap(llrs, "llrs")
    r = _device.wrap(reference, "reference")
    if x.shape != r.shape:
        raise ValueError(f"{name}: llrs {x.shape} and reference {r.shape} differ in shape.")
    if x.ndim not in (1, 2):
        raise ValueError(f"{name}: llrs must be 1-D or 2-D, got {x.ndim}-D.")
    k = constellation.bits_per_symbol
    if x.shape[-1] % k:
        raise ValueError(f"{name}: the last axis ({x.shape[-1]}) is not a multiple of bits_per_symbol ({k}).")
    skip = int(num_skip_symbols) * k
    if skip < 0 or skip >= x.shape[-1]:
        raise ValueError(f"{name}: num_skip_symbols leaves no LLRs.")
    import torch

    if x.kind != "torch":
        llrs, reference = torch.as_tensor(llrs, device=f"cuda:{x.device}"), torch.as_tensor(
            reference, device=f"cuda:{x.device}")  # fmt: skip
    was_1d = x.ndim == 1
    L = llrs.reshape(1, -1) if was_1d else llrs
    c = reference.reshape(1, -1) if was_1d else reference
    L = L[:, skip:].to(torch.float32).contiguous()
    c = (c[:, skip:] != 0).to(torch.int8).contiguous()
    rows, length = L.shape
    chunks = (length + _lib.CK_GMI_CHUNK - 1) // _lib.CK_GMI_CHUNK
    partial = torch.empty((rows, chunks), dtype=torch.float64, device=L.device)
    ld = _device.wrap(L)
    with _device.on_device(ld):
        st = _lib.lib().ck_gmi_loss(ld.ptr, c.data_ptr(), rows, length, partial.data_ptr(), _device.stream_of(ld))
        _lib.check(st, name)
    loss = partial.sum(dim=1) / length
    return loss, constellation, was_1d


def _report(v: Any, was_1d: bool) -> float | np.ndarray:
    out = v.cpu().numpy()
    return float(out[0]) if was_1d else out


def _array_only(noise_var: Any, esn0_db: Any, name: str) -> None:
    """``noise_var``/``esn0_db`` demap a Signal's symbols in the reference;
    LLR arrays already contain the noise (``commkit/metrics/information.py:
    64-68``)."""
    if noise_var is not None or esn0_db is not None:
        raise ValueError(f"{name}: noise_var and esn0_db are for Signal input; LLR arrays "
                         "already contain the noise.")  # fmt: skip


def gmi(llrs: Any, reference: Any = None, *, constellation: Constellation | None = None,
        noise_var: float | None = None, esn0_db: float | None = None, method: str = "maxlog",
        num_skip_symbols: int = 0) -> float | np.ndarray:  # fmt: skip
    """Generalized mutual information in bits per symbol
    (``commkit/metrics/information.py:90-166``): ``H(X) - sum_b E[log2(1 +
    e^{-(1-2c_b) L_b})]`` for LLRs ``(N k,)`` (a float) or ``(C, N k)``
    (``(C,)``) on a CUDA device, with the transmitted ``reference`` bits.
    ``noise_var``, ``esn0_db`` and ``method`` belong to the reference's
    Signal input (received symbols), which this package does not take: with
    an LLR array, ``noise_var``/``esn0_db`` raise ``ValueError`` as there."""
    _array_only(noise_var, esn0_db, "gmi()")
    loss, c, was_1d = _loss(llrs, reference, constellation, num_skip_symbols, "gmi()")
    k = c.bits_per_symbol
    return _report(k * (c.entropy / k - loss), was_1d)


def ngmi(llrs: Any, reference: Any = None, *, constellation: Constellation | None = None,
         noise_var: float | None = None, esn0_db: float | None = None, method: str = "maxlog",
         num_skip_symbols: int = 0) -> float | np.ndarray:  # fmt: skip
    """Normalized GMI, ``1 - loss`` (``commkit/metrics/information.py:169-236``);
    the arguments as for :func:`gmi`."""
    _array_only(noise_var, esn0_db, "ngmi()")
    loss, _, was_1d = _loss(llrs, reference, constellation, num_skip_symbols, "ngmi()")
    return _report(1.0 - loss, was_1d)
