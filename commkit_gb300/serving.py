"""A continuous-batching request loop for demap + decode.

Requests carry frames of one code on one constellation with one Es/N0.
They arrive over time (:func:`poisson_requests` draws a seeded stream). The
:class:`Server` keeps LLRs and check-message state on the device and admits
requests whenever the device memory they need fits the HBM budget and a
batch slot is free. Each batch takes everything admitted since the previous
one, demaps it per (code, constellation) and decodes every code in ONE
launch of the mixed-code persistent kernel. Each batch runs on its own
CUDA stream, so a batch admitted while others are still on the GPU overlaps
with them; when a batch completes, its memory returns to the budget. Per
request the server records the latency from arrival to results in host
memory.

The admission and batching policy (:class:`Admission`) is plain Python and
is tested without a GPU.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from .coding import LDPCCode, MinSum, decode_mixed
from .mapping import Constellation, compute_llr_frames, inv_s2_frames


@dataclass
class Request:
    """Frames of one code on one constellation at one Es/N0."""

    rid: int
    code: str
    order: int
    symbols: Any  # (F, S) complex64, host (ideally pinned)
    noise_var: float
    arrival: float = 0.0  # seconds from the stream's start
    # filled by the server
    admitted: float = float("nan")
    done: float = float("nan")
    bits: Any = None
    llrs: Any = None
    valid: Any = None
    iterations: Any = None

    @property
    def frames(self) -> int:
        return int(self.symbols.shape[0])

    @property
    def latency(self) -> float:
        return self.done - self.arrival


@dataclass
class Admission:
    """Admission against a device-memory budget and a limit on batches in flight.

    ``cost(request)`` is the device bytes a request holds from admission to
    completion; ``batch_overhead`` the bytes each batch adds (its decoder
    workspace).  Requests are admitted in arrival order (no overtaking), as
    many as fit when a batch slot is free.
    """

    budget: int
    max_inflight: int
    batch_overhead: int = 0
    max_batch_frames: int = 1 << 20
    in_use: int = 0
    inflight: int = 0
    pending: deque = field(default_factory=deque)

    def arrive(self, req: Request) -> None:
        self.pending.append(req)

    def next_batch(self, cost) -> list[Request]:
        """The requests of the next batch (possibly none), charged to the budget."""
        if self.inflight >= self.max_inflight or not self.pending:
            return []
        batch, spent, frames = [], self.batch_overhead, 0
        while self.pending:
            r = self.pending[0]
            c = cost(r)
            if self.in_use + spent + c > self.budget or frames + r.frames > self.max_batch_frames:
                break
            batch.append(self.pending.popleft())
            spent += c
            frames += r.frames
        if not batch:
            if self.in_use == 0 and self.inflight == 0:
                raise MemoryError(
                    f"request {self.pending[0].rid} needs {cost(self.pending[0]) + self.batch_overhead} bytes, "
                    f"more than the {self.budget}-byte budget"
                )
            return []
        self.in_use += spent
        self.inflight += 1
        return batch

    def release(self, spent: int) -> None:
        self.in_use -= spent
        self.inflight -= 1


class Server:
    """Demap + decode server on one CUDA device (see the module docstring)."""

    def __init__(self, codes: dict[str, LDPCCode], method: MinSum, *, hbm_budget: int = 4 << 30,
                 max_inflight: int = 3, device: Any = None):  # fmt: skip
        import torch

        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.codes = codes
        self.method = method
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max_inflight)]
        self._next_stream = 0
        # The decoder workspace of a batch: the device-memory message slots
        # of the largest code for a full grid, plus the header.
        ws = 256
        for code in codes.values():
            plan = code._plan(self.device.index)
            ws = max(ws, plan.workspace_size(1 << 20))
        self.admission = Admission(budget=hbm_budget, max_inflight=max_inflight, batch_overhead=ws)
        self.inflight: list[tuple] = []
        self.completed: list[Request] = []

    def cost(self, r: Request) -> int:
        """Device bytes a request holds: symbols, inverse noise variances, LLRs,
        a-posteriori LLRs, bits and flags."""
        code = self.codes[r.code]
        return r.frames * (r.symbols.shape[1] * 8 + 4 + 8 * code.n + code.k + 5)

    def _launch(self, batch: list[Request], t0: float) -> None:
        torch = self.torch
        stream = self.streams[self._next_stream]
        self._next_stream = (self._next_stream + 1) % len(self.streams)
        now = time.perf_counter() - t0
        for r in batch:
            r.admitted = now
        keep = []
        with torch.cuda.stream(stream):
            per_code: dict[str, list[Request]] = {}
            for r in batch:
                per_code.setdefault(r.code, []).append(r)
            jobs, layout = [], []
            for name, rs in per_code.items():
                code = self.codes[name]
                total = sum(r.frames for r in rs)
                llr = torch.empty((total, code.n), dtype=torch.float32, device=self.device)
                off = 0
                by_order: dict[int, list[Request]] = {}
                for r in rs:
                    by_order.setdefault(r.order, []).append(r)
                for order, group in by_order.items():
                    frames = sum(r.frames for r in group)
                    sym = torch.empty((frames, group[0].symbols.shape[1]), dtype=torch.complex64, device=self.device)
                    s2 = np.empty(frames, np.float32)
                    o = 0
                    for r in group:
                        src = r.symbols if isinstance(r.symbols, torch.Tensor) else torch.from_numpy(r.symbols)
                        sym[o : o + r.frames].copy_(src, non_blocking=True)
                        s2[o : o + r.frames] = inv_s2_frames([r.noise_var])[0]
                        o += r.frames
                    s2_dev = torch.from_numpy(s2).pin_memory().to(self.device, non_blocking=True)
                    compute_llr_frames(sym, constellation=Constellation.qam(order), inv_s2=s2_dev,
                                       out=llr[off : off + frames])  # fmt: skip
                    keep += [sym, s2_dev]
                    for r in group:
                        layout.append((r, name, off))
                        off += r.frames
                jobs.append((llr, code, self.method))
                keep.append(llr)
            results = decode_mixed(jobs)
            host = {}
            for (llr, code, _), (name, res) in zip(jobs, zip(per_code, results, strict=True), strict=True):
                h = tuple(torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in
                          (res.bits, res.llrs, res.valid, res.iterations))  # fmt: skip
                for a, b in zip(h, (res.bits, res.llrs, res.valid, res.iterations), strict=True):
                    a.copy_(b, non_blocking=True)
                host[name] = h
                keep.append(res)
            event = torch.cuda.Event()
            event.record(stream)
        spent = sum(self.cost(r) for r in batch) + self.admission.batch_overhead
        self.inflight.append((event, batch, layout, host, keep, spent))

    def _poll(self, t0: float, block: bool = False) -> None:
        still = []
        for item in self.inflight:
            event, batch, layout, host, keep, spent = item
            if not (event.query() or (block and (event.synchronize() or True))):
                still.append(item)
                continue
            now = time.perf_counter() - t0
            for r, name, off in layout:
                bits, llrs, valid, iters = host[name]
                sl = slice(off, off + r.frames)
                r.bits, r.llrs = bits[sl].numpy(), llrs[sl].numpy()
                r.valid, r.iterations = valid[sl].numpy(), iters[sl].numpy()
                r.done = now
                self.completed.append(r)
            self.admission.release(spent)
        self.inflight = still

    def serve(self, requests: list[Request], *, spin: float = 20e-6) -> list[Request]:
        """Run a request stream (arrival times in seconds from now) to completion."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        self.completed = []
        t0 = time.perf_counter()
        while pending or self.admission.pending or self.inflight:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                self.admission.arrive(pending.popleft())
            self._poll(t0)
            batch = self.admission.next_batch(self.cost)
            if batch:
                self._launch(batch, t0)
                continue
            if not self.admission.pending and not pending and self.inflight:
                time.sleep(spin)
            elif pending and not self.admission.pending and not self.inflight:
                time.sleep(max(0.0, min(pending[0].arrival - now, 1e-3)))
            else:
                time.sleep(spin)
        self._poll(t0, block=True)
        return self.completed


# ---------------------------------------------------------------------------
# Seeded request streams
# ---------------------------------------------------------------------------

# Es/N0 (dB) at FER ~ 0.5 of each (code, constellation), MinSum 50 iterations,
# measured with this package's decoder: the request stream sits around them.
WATERFALL_ESN0_DB = {
    ("A", 4): 1.15, ("A", 16): 6.4, ("A", 64): 10.9,
    ("B", 4): 4.1, ("B", 16): 10.1, ("B", 64): 15.5,
    ("C", 4): 0.35, ("C", 16): 5.35, ("C", 64): 9.25,
}  # fmt: skip


@dataclass
class PayloadPool:
    """Pre-generated received frames per (code, constellation), so a stream
    of requests costs no encoding or noise generation while it runs."""

    frames: dict  # (code, order) -> (symbols (F, S) complex64, esn0 (F,))

    @classmethod
    def build(cls, frames_per_pool: dict, seed: int = 0, spread_db: float = 1.0, pinned: bool = True):
        import torch

        from . import workloads as W

        rng = np.random.default_rng(seed)
        pools = {}
        for (name, order), n in frames_per_pool.items():
            spec = W.CODES[name]
            esn0 = WATERFALL_ESN0_DB[(name, order)] + rng.uniform(-spread_db, spread_db, n)
            R = (spec.nb - spec.mb) / spec.nb
            k = int(round(np.log2(order)))
            ebn0 = esn0 - 10.0 * np.log10(R * k)
            b = W.coded_batch(spec, n, order, ebn0, seed=int(rng.integers(2**31)))
            sym = torch.from_numpy(b.symbols)
            pools[(name, order)] = (sym.pin_memory() if pinned else sym, b.noise_var)
        return cls(pools)


def poisson_requests(rate_hz: float, duration_s: float, pool: PayloadPool, *, mix=(0.5, 0.35, 0.15),
                     orders=(4, 16, 64), max_frames: int = 256, seed: int = 0) -> list[Request]:  # fmt: skip
    """Poisson arrivals at ``rate_hz`` for ``duration_s``: each request takes
    1..``max_frames`` frames (log-uniform) of code A/B/C (``mix``) on a random
    constellation of ``orders``, one Es/N0 (the pool frames' own noise
    variance of its first frame, all its frames drawn near the waterfall)."""
    rng = np.random.default_rng(seed)
    t, rid, out = 0.0, 0, []
    names = ("A", "B", "C")
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            break
        name = names[rng.choice(3, p=np.asarray(mix) / np.sum(mix))]
        order = int(orders[rng.integers(len(orders))])
        if (name, order) not in pool.frames:
            order = next(o for o in orders if (name, o) in pool.frames)
        frames = int(np.clip(np.round(np.exp(rng.uniform(0.0, np.log(max_frames)))), 1, max_frames))
        sym, nv = pool.frames[(name, order)]
        start = int(rng.integers(0, max(1, sym.shape[0] - frames + 1)))
        frames = min(frames, sym.shape[0])
        out.append(Request(rid, name, order, sym[start : start + frames], float(nv[start]), arrival=t))
        rid += 1
    return out
