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
is tested without a GPU.  Each batch slot holds preallocated device buffers
and pinned staging, so a batch costs one host-to-device copy of its
symbols, one of its inverse noise variances, a demap launch per (code,
constellation), one decode launch and one device-to-host copy per output,
all on the slot's stream, with no allocation.
"""

from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field
from typing import Any

import numpy as np

import ctypes

from . import _lib
from .coding import LDPCCode, MinSum
from .mapping import Constellation, inv_s2_frames


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
    """FIFO admission into a fixed number of batch slots.

    Each slot's device memory is allocated once, when the server starts, so
    the HBM budget is ``slots x bytes per slot``; a batch is whatever
    arrived requests fit one slot (``fits(batch, request)``: the slot's
    per-code frame and symbol capacities).  Requests are admitted in arrival
    order (no overtaking), as many as fit, whenever a slot is free.
    """

    slots: int
    free: int = -1
    pending: deque = field(default_factory=deque)

    def __post_init__(self) -> None:
        if self.free < 0:
            self.free = self.slots

    def arrive(self, req: Request) -> None:
        self.pending.append(req)

    def next_batch(self, fits) -> list[Request]:
        """The requests of the next batch (possibly none); takes a slot."""
        if self.free <= 0 or not self.pending:
            return []
        batch: list[Request] = []
        while self.pending and fits(batch, self.pending[0]):
            batch.append(self.pending.popleft())
        if not batch:
            raise MemoryError(f"request {self.pending[0].rid} does not fit an empty batch slot")
        self.free -= 1
        return batch

    def release(self) -> None:
        self.free += 1


class _Slot:
    """One batch slot: device buffers, pinned staging and a stream."""

    def __init__(self, server: Server, caps: dict[str, int], sym_bytes: int):
        torch = server.torch
        dev = server.device
        self.stream = torch.cuda.Stream(dev)
        self.caps = caps
        total = sum(caps.values())
        self.sym_dev = torch.empty(sym_bytes // 8, dtype=torch.complex64, device=dev)
        self.s2_dev = torch.empty(total, dtype=torch.float32, device=dev)
        self.s2_host = torch.empty(total, dtype=torch.float32, pin_memory=True)
        self.llr, self.out_dev, self.out_host = {}, {}, {}
        for name, cap in caps.items():
            code = server.codes[name]
            self.llr[name] = torch.empty((cap, code.n), dtype=torch.float32, device=dev)
            shapes = (((cap, code.n), torch.float32), ((cap, code.k), torch.int8), ((cap,), torch.int32),
                      ((cap,), torch.uint8))  # fmt: skip
            self.out_dev[name] = [torch.empty(sh, dtype=dt, device=dev) for sh, dt in shapes]
        arr = server._batch_array({name: (cap, self) for name, cap in caps.items()})
        need = ctypes.c_size_t(0)
        _lib.check(_lib.lib().ck_ldpc_mixed_workspace_size(arr, len(caps), ctypes.byref(need)), "server slot")
        self.ws = torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=dev)
        self.bytes = (self.sym_dev.numel() * 8 + self.s2_dev.numel() * 4 + self.ws.numel()
                      + sum(t.numel() * t.element_size() for v in self.out_dev.values() for t in v)
                      + sum(t.numel() * 4 for t in self.llr.values()))  # fmt: skip
        self.event = torch.cuda.Event()
        self.batch: list = []
        self.layout: list = []
        self.counts: dict[str, int] = {}


class Server:
    """Demap + decode server on one CUDA device (see the module docstring).

    ``frames_per_slot`` caps each code's frames in one batch; the slots'
    device memory (``slots`` of them) must fit ``hbm_budget``.
    """

    def __init__(self, codes: dict[str, LDPCCode], method: MinSum, *, hbm_budget: int = 4 << 30,
                 max_inflight: int = 3, device: Any = None, frames_per_slot: dict | None = None,
                 orders=(4, 16, 64)):  # fmt: skip
        import torch

        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.codes = codes
        self.method = method
        self.orders = tuple(orders)
        # Symbols of a full slot at the densest constellation (fewest bits per symbol).
        kmin = min(int(round(np.log2(o))) for o in self.orders)
        if frames_per_slot is None:
            # An equal share of the budget per slot and code, less a decoder
            # workspace (the largest code's full-grid message state).
            ws = max(code._plan(self.device.index).workspace_size(1 << 20) for code in codes.values())
            share = max(0, hbm_budget // max_inflight - ws) // len(codes)
            frames_per_slot = {}
            for name, code in codes.items():
                per_frame = (code.n // kmin) * 8 + 4 + 8 * code.n + code.k + 8
                frames_per_slot[name] = max(1, int(share // per_frame))
        self.caps = {name: int(frames_per_slot[name]) for name in codes}
        sym_bytes = sum(cap * (codes[n].n // kmin) * 8 for n, cap in self.caps.items())
        self._sym_cap = sym_bytes // 8
        with torch.cuda.device(self.device):
            self._tables = {o: self._axis_structs(o) for o in self.orders}
            self.slots = [_Slot(self, self.caps, sym_bytes) for _ in range(max_inflight)]
        used = sum(sl.bytes for sl in self.slots)
        if used > hbm_budget:
            raise MemoryError(f"{max_inflight} batch slots need {used} bytes, over the {hbm_budget}-byte budget")
        self.hbm_bytes = used
        self.admission = Admission(slots=max_inflight)
        self._free = list(self.slots)
        self._busy: list[_Slot] = []
        self.completed: list[Request] = []

    def _axis_structs(self, order: int):
        from . import _device
        from .mapping import _axis_struct, device_tables

        like = _device.wrap(self.torch.empty(1, device=self.device))
        tabs = device_tables(Constellation.qam(order), "maxlog", like)
        half = len(tabs) // 2
        return (_axis_struct(tabs[:half], "maxlog"), _axis_struct(tabs[half:], "maxlog"), tabs)

    def _batch_array(self, counts: dict):
        arr = (_lib.Batch * len(counts))()
        m = self.method
        for i, (name, (B, slot)) in enumerate(counts.items()):
            code = self.codes[name]
            o = slot.out_dev[name]
            arr[i] = _lib.Batch(code._plan(self.device.index).handle, slot.llr[name].data_ptr(), o[0].data_ptr(), B,
                                code.n, _lib.CK_LDPC_MIN_SUM, np.float32(m.scale), np.float32(m.offset),
                                int(m.max_iterations), 1 if m.early_stop else 0, o[2].data_ptr(),
                                o[3].data_ptr(), o[1].data_ptr(), code.k)  # fmt: skip
        return arr

    def _fits(self, batch: list[Request], r: Request) -> bool:
        frames = sum(q.frames for q in batch if q.code == r.code) + r.frames
        syms = sum(q.frames * q.symbols.shape[1] for q in batch) + r.frames * r.symbols.shape[1]
        return frames <= self.caps[r.code] and syms <= self._sym_cap

    def _launch(self, batch: list[Request], t0: float) -> None:
        torch = self.torch
        slot = self._free.pop()
        now = time.perf_counter() - t0
        slot.batch, slot.layout = batch, []
        groups: dict[tuple[str, int], list[Request]] = {}
        for r in batch:
            r.admitted = now
            groups.setdefault((r.code, r.order), []).append(r)
        s2_np = slot.s2_host.numpy()
        sym_off, s2_off, counts, demaps, copies = 0, 0, {}, [], []
        for name in self.codes:
            frame_off = 0
            for order in self.orders:
                group = groups.get((name, order))
                if not group:
                    continue
                S = group[0].symbols.shape[1]
                g_frames = sum(r.frames for r in group)
                g_sym = sym_off
                for r in group:
                    # Each request's (pinned) symbols go straight to the device.
                    copies.append((sym_off, r.frames * S, r.symbols))
                    s2_np[s2_off : s2_off + r.frames] = inv_s2_frames([r.noise_var])[0]
                    slot.layout.append((r, name, frame_off))
                    sym_off += r.frames * S
                    s2_off += r.frames
                    frame_off += r.frames
                demaps.append((order, g_sym, S, g_frames, s2_off - g_frames, name, frame_off - g_frames))
            if frame_off:
                counts[name] = frame_off
        slot.counts = counts
        lib = _lib.lib()
        with torch.cuda.stream(slot.stream):
            for off, n, src in copies:
                if not isinstance(src, torch.Tensor):
                    src = torch.from_numpy(np.ascontiguousarray(src))
                slot.sym_dev[off : off + n].copy_(src.reshape(-1), non_blocking=True)
            slot.s2_dev[:s2_off].copy_(slot.s2_host[:s2_off], non_blocking=True)
            st = slot.stream.cuda_stream
            for order, g_sym, S, g_frames, g_s2, name, f_off in demaps:
                re, im, _ = self._tables[order]
                x_ptr = slot.sym_dev.data_ptr() + 8 * g_sym
                out_ptr = slot.llr[name].data_ptr() + 4 * f_off * self.codes[name].n
                _lib.check(lib.ck_llr_separable_maxlog_frames(
                    x_ptr, g_frames * S, S, slot.s2_dev.data_ptr() + 4 * g_s2, ctypes.byref(re), ctypes.byref(im),
                    out_ptr, st), "server demap")  # fmt: skip
            arr = self._batch_array({name: (B, slot) for name, B in counts.items()})
            _lib.check(lib.ck_ldpc_decode_mixed(arr, len(counts), slot.ws.data_ptr(), slot.ws.numel(), st),
                       "server decode")  # fmt: skip
            # Results land in pinned buffers of this batch, which the requests
            # then view (no host-side copies).
            slot.out_host = {}
            for name, B in counts.items():
                hs = []
                for d in slot.out_dev[name]:
                    h = torch.empty((B, *d.shape[1:]), dtype=d.dtype, pin_memory=True)
                    h.copy_(d[:B], non_blocking=True)
                    hs.append(h)
                slot.out_host[name] = hs
            slot.event.record(slot.stream)
        self._busy.append(slot)

    def _poll(self, t0: float, block: bool = False) -> None:
        still = []
        for slot in self._busy:
            if not slot.event.query():
                if not block:
                    still.append(slot)
                    continue
                slot.event.synchronize()
            now = time.perf_counter() - t0
            for r, name, off in slot.layout:
                llrs, bits, iters, valid = (t.numpy() for t in slot.out_host[name])
                sl = slice(off, off + r.frames)
                r.bits, r.llrs, r.iterations = bits[sl], llrs[sl], iters[sl]
                r.valid = valid[sl].view(np.bool_)
                r.done = now
                self.completed.append(r)
            slot.batch, slot.layout = [], []
            self._free.append(slot)
            self.admission.release()
        self._busy = still

    def serve(self, requests: list[Request]) -> list[Request]:
        """Run a request stream (arrival times in seconds from now) to completion."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        self.completed = []
        t0 = time.perf_counter()
        while pending or self.admission.pending or self._busy:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                self.admission.arrive(pending.popleft())
            if self._busy:
                self._poll(t0)
            batch = self.admission.next_batch(self._fits)
            if batch:
                self._launch(batch, t0)
            elif pending and not self.admission.pending and not self._busy:
                wait = pending[0].arrival - (time.perf_counter() - t0)
                if wait > 2e-4:
                    time.sleep(wait - 1e-4)
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
