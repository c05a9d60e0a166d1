"""Error-rate curves of an LDPC code over AWGN, simulated on the device:
:func:`error_rate_curve` and :class:`ErrorRateCurve`.

``commkit/coding/performance.py:43-352``.  At each Es/N0 the coded link runs
in batches until ``min_block_errors`` block errors or ``max_blocks`` blocks:
random information bits, :func:`~commkit_gb300.coding.encode`, the
constellation's points plus AWGN, :func:`~commkit_gb300.compute_llr` and
:func:`~commkit_gb300.decode`, then the counts.  Every step is a kernel on
the batch's device (``csrc/ck_sim.cu`` for the bits, the encoder, the
mapping, the noise and the counts); the only transfer per batch is the
device-to-host copy of the seven counters that decides whether the point
stops.

The reference draws the information bits on the host and the noise with
the array library's generator; here both come from one counter-based
generator (Philox-4x32-10) keyed by ``rng``, so a curve is reproducible for
a seed, on any launch shape.  The counts have the reference's meaning.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _device, _lib
from .coding import LDPCCode, MinSum, SumProduct, _resolve_method, decode, encode_blocks
from .mapping import Constellation

__all__ = ["ErrorRateCurve", "error_rate_curve"]

# Transmitted bits per batch (the reference's _BATCH_BITS,
# commkit/coding/performance.py:38).
BATCH_BITS = 1 << 18

_COUNT_FIELDS = (
    "num_blocks",
    "bit_errors",
    "block_errors",
    "pre_fec_bit_errors",
    "detected_failures",
    "undetected_errors",
    "total_iterations",
)


@dataclass(frozen=True, eq=False)
class ErrorRateCurve:
    """Decoding error counts of a code against Es/N0, one entry per point
    (``commkit/coding/performance.py:43-169``)."""

    esn0_db: np.ndarray
    num_blocks: np.ndarray
    bit_errors: np.ndarray
    block_errors: np.ndarray
    pre_fec_bit_errors: np.ndarray
    detected_failures: np.ndarray
    undetected_errors: np.ndarray
    total_iterations: np.ndarray
    k: int
    n: int
    bits_per_symbol: int
    checked: bool = True
    label: str = ""

    def __post_init__(self) -> None:
        esn0 = np.array(self.esn0_db, dtype=np.float64)
        if esn0.ndim != 1 or esn0.size == 0 or not np.all(np.isfinite(esn0)):
            raise ValueError(f"ErrorRateCurve: esn0_db must be 1-D, finite and not empty, got shape {esn0.shape}.")
        esn0.setflags(write=False)
        object.__setattr__(self, "esn0_db", esn0)
        for name in _COUNT_FIELDS:
            v = np.asarray(getattr(self, name))
            if v.shape != esn0.shape:
                raise ValueError(f"ErrorRateCurve: {name} must have the shape of esn0_db {esn0.shape}, got {v.shape}.")
            if v.dtype.kind not in "iu" or np.any(v < 0):
                raise ValueError(f"ErrorRateCurve: {name} must be counts >= 0.")
            v = v.astype(np.int64)
            v.setflags(write=False)
            object.__setattr__(self, name, v)
        if np.any(self.num_blocks < 1):
            raise ValueError("ErrorRateCurve: num_blocks must be >= 1 at every point.")
        for name in ("k", "n", "bits_per_symbol"):
            v = getattr(self, name)
            if isinstance(v, bool) or not isinstance(v, (int, np.integer)) or v < 1:
                raise ValueError(f"ErrorRateCurve: {name} must be an integer >= 1, got {v!r}.")
            object.__setattr__(self, name, int(v))
        object.__setattr__(self, "checked", bool(self.checked))

    @property
    def rate(self) -> float:
        return self.k / self.n

    @property
    def ebn0_db(self) -> np.ndarray:
        return self.esn0_db - 10 * np.log10(self.rate * self.bits_per_symbol)

    @property
    def ber(self) -> np.ndarray:
        return self.bit_errors / (self.num_blocks * self.k)

    @property
    def fer(self) -> np.ndarray:
        return self.block_errors / self.num_blocks

    @property
    def pre_fec_ber(self) -> np.ndarray:
        return self.pre_fec_bit_errors / (self.num_blocks * self.n)

    @property
    def mean_iterations(self) -> np.ndarray:
        return self.total_iterations / self.num_blocks


def _seed_of(rng: Any) -> int:
    if rng is None:
        return int(np.random.default_rng().integers(0, 2**63))
    if isinstance(rng, np.random.Generator):
        return int(rng.integers(0, 2**63))
    if isinstance(rng, (int, np.integer)) and not isinstance(rng, bool):
        return int(np.random.default_rng(int(rng)).integers(0, 2**63))
    raise TypeError(f"rng must be an int, a numpy Generator or None, got {type(rng).__name__}.")


@dataclass
class LinkBatch:
    """Device buffers of one batch of ``blocks`` codewords and the steps that
    fill them: ``info`` (blocks, k), ``record`` (the codewords then filler
    bits up to whole symbols), ``symbols``, ``llrs`` (blocks, n), the
    decoder's result and ``counts`` (7,) int64."""

    code: LDPCCode
    constellation: Constellation
    method: MinSum | SumProduct
    blocks: int
    device: Any
    seed: int
    buffers: dict = field(default_factory=dict)

    def __post_init__(self) -> None:
        import torch

        code, c = self.code, self.constellation
        kb = c.bits_per_symbol
        bits = self.blocks * code.n
        self.n_sym = -(-bits // kb)
        dev = torch.device(self.device)
        self.torch = torch
        self.info = torch.empty((self.blocks, code.k), dtype=torch.int8, device=dev)
        self.record = torch.empty(self.n_sym * kb, dtype=torch.int8, device=dev)
        self.words = self.record[:bits].view(self.blocks, code.n)
        self.symbols = torch.empty(self.n_sym, dtype=torch.complex64, device=dev)
        self.counts = torch.zeros(len(_COUNT_FIELDS), dtype=torch.int64, device=dev)
        by_label = np.empty(c.order, dtype=np.complex64)
        from .mapping import _packed

        by_label[_packed(c.bit_labels)] = c.points.astype(np.complex64)
        self.points = torch.from_numpy(by_label).to(dev)
        self.scratch = torch.empty(code._encoder.scratch_bytes(self.blocks, code.num_checks, code.k),
                                   dtype=torch.int8, device=dev)
        self.ws = torch.empty(max(code._plan(dev.index).workspace_size(
            self.blocks, _lib.CK_LDPC_SUM_PRODUCT if isinstance(self.method, SumProduct) else _lib.CK_LDPC_MIN_SUM),
            256), dtype=torch.uint8, device=dev)  # fmt: skip
        self.result = None
        self.llrs = None

    def run(self, noise_var: float, stream_id: int, blocks: int | None = None) -> None:
        """One batch at ``noise_var`` (the variance of the noise in the
        symbols, as :func:`compute_llr` takes it), Philox streams
        ``2 stream_id`` (bits) and ``2 stream_id + 1`` (noise); ``blocks``
        may cut the batch short.  Adds to :attr:`counts`."""
        torch = self.torch
        code, c = self.code, self.constellation
        b = self.blocks if blocks is None else int(blocks)
        kb = c.bits_per_symbol
        bits = b * code.n
        n_sym = -(-bits // kb)
        lib = _lib.lib()
        dev = _device.wrap(self.info)
        st = _device.stream_of(dev)
        with _device.on_device(dev):
            info = self.info[:b]
            _lib.check(lib.ck_random_bits(info.data_ptr(), b * code.k, self.seed, 2 * stream_id, st), "random bits")
            words = self.record[:bits].view(b, code.n)
            encode_blocks(code, info, words, self.scratch)
            if n_sym * kb > bits:  # filler bits up to whole symbols
                _lib.check(lib.ck_random_bits(self.record.data_ptr() + bits, n_sym * kb - bits, self.seed,
                                              2 * stream_id + 1 + (1 << 62), st), "filler bits")  # fmt: skip
            if c.is_complex:
                std_re = std_im = math.sqrt(noise_var / 2)
                nv_llr = noise_var
            else:
                # Real noise of variance noise_var on the in-phase axis only; the
                # complex symbols' LLRs then take twice it, as real input does.
                std_re, std_im, nv_llr = math.sqrt(noise_var), 0.0, 2.0 * noise_var
            sym = self.symbols[:n_sym]
            _lib.check(lib.ck_map_awgn(self.record.data_ptr(), n_sym, kb, self.points.data_ptr(), std_re, std_im,
                                       self.seed, 2 * stream_id + 1, sym.data_ptr(), st), "map/AWGN")  # fmt: skip
            llrs = c.llr(sym, noise_var=nv_llr).reshape(-1)[:bits].view(b, code.n)
            res = decode(llrs, code=code, method=self.method, workspace=self.ws)
            dec_bits = res.bits.reshape(b, code.k)
            valid = res.valid.reshape(b).view(torch.uint8)
            iters = res.iterations.reshape(b)
            _lib.check(lib.ck_count_errors(info.data_ptr(), dec_bits.data_ptr(), llrs.data_ptr(), words.data_ptr(),
                                           b, code.k, code.n, valid.data_ptr(), iters.data_ptr(),
                                           self.counts.data_ptr(), st), "error counts")  # fmt: skip
        self.llrs, self.result = llrs, res


def error_rate_curve(code: LDPCCode, *, constellation: Constellation, esn0_db: Any, method: Any = None,
                     min_block_errors: int = 100, max_blocks: int = 10_000, label: str | None = None,
                     rng: Any = None, device: Any = None, batch_blocks: int | None = None) -> ErrorRateCurve:  # fmt: skip
    """Measure an LDPC code's error rates over AWGN by Monte Carlo on a CUDA
    device (``commkit/coding/performance.py:172-352``).

    ``esn0_db`` ``(P,)``; each point runs batches (``batch_blocks``, by
    default about 2^18 transmitted bits, at least one block) until
    ``min_block_errors`` blocks are in error or ``max_blocks`` blocks are
    decoded.  The noise is circular complex of variance ``N0 = Es/(Es/N0)``
    for a complex constellation, real of variance ``N0/2`` for a real one,
    and the LLRs use it and the constellation's prior.  ``device``: a CUDA
    device (the current one by default).
    """
    import torch

    name = "error_rate_curve()"
    if not isinstance(code, LDPCCode):
        raise TypeError(f"{name}: code must be an LDPCCode, got {type(code).__name__}.")
    method = _resolve_method(method)
    if not isinstance(constellation, Constellation):
        raise TypeError(f"{name}: constellation must be a Constellation, got {type(constellation).__name__}.")
    if constellation.pmf is not None:
        raise ValueError(f"{name}: a shaped constellation with a FEC code needs a distribution matcher, "
                         "which this package does not provide.")  # fmt: skip
    grid = np.array(esn0_db, dtype=np.float64).reshape(-1) if np.ndim(esn0_db) <= 1 else None
    if grid is None or grid.size == 0 or not np.all(np.isfinite(grid)):
        raise ValueError(f"{name}: esn0_db must be 1-D, finite and not empty.")
    for arg, v in (("min_block_errors", min_block_errors), ("max_blocks", max_blocks)):
        if isinstance(v, bool) or not isinstance(v, (int, np.integer)) or v < 1:
            raise ValueError(f"{name}: {arg} must be an integer >= 1, got {v!r}.")
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    if dev.type != "cuda":
        raise ValueError(f"{name}: device must be a CUDA device, got {dev}.")
    batch = int(batch_blocks) if batch_blocks else max(1, -(-BATCH_BITS // code.n))
    link = LinkBatch(code, constellation, method, batch, dev, _seed_of(rng))
    es = constellation.power()
    counts = np.zeros((len(_COUNT_FIELDS), grid.size), dtype=np.int64)
    stream = 0
    for i, esn0 in enumerate(grid):
        n0 = es / 10 ** (esn0 / 10)
        noise_var = n0 if constellation.is_complex else n0 / 2
        link.counts.zero_()
        while counts[0, i] < max_blocks and counts[2, i] < min_block_errors:
            b = int(min(batch, max_blocks - counts[0, i]))
            link.run(noise_var, stream, b)
            stream += 1
            counts[:, i] = link.counts.cpu().numpy()  # the one transfer of the batch
    if label is None:
        label = f"{type(method).__name__} on {code!r}"
    return ErrorRateCurve(grid, **dict(zip(_COUNT_FIELDS, counts, strict=True)), k=code.k, n=code.n,
                          bits_per_symbol=constellation.bits_per_symbol, checked=True, label=label)  # fmt: skip
