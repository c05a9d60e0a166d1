"""A continuous-batching request loop for demap + decode.

Requests carry frames of one code on one constellation with one Es/N0.
They arrive over time (:func:`poisson_requests` draws a seeded stream).
The :class:`Server` keeps LLRs and check-message state on the device and
admits requests whenever a batch slot is free; a slot's device memory is
allocated once, so the HBM budget is ``slots x bytes per slot``.  Each
batch takes the arrived requests that fit one slot and decodes them in ONE
launch of the mixed-code persistent kernel, one batch entry per (code,
constellation), which demaps each frame as it loads it; on the slot's own
CUDA stream: batches admitted while others run overlap with them on the
device.

Zero-copy on GB300: the Grace host memory is coherent with the GPU over
NVLink-C2C and pinned allocations have one address on both sides.  So a
batch is assembled by one gather kernel that reads every request's pinned
symbols (and the frames' noise scales) in place, and the decoder writes
each frame's a-posteriori LLRs, bits, iterations and syndrome flag straight
into a pinned output arena.  A batch costs one gather launch, one decode
launch and an event: no per-request copy call, no device-to-host copy, no
allocation.  (Where a constellation's demapping cannot run inside the
decoder, a demap launch per (code, constellation) fills LLR buffers first.)

The arena is a ring: request results (:attr:`Request.llrs` etc.) are views
into it and stay valid until ``output_arena_bytes`` of later results have
been written; copy them out to keep them longer.  Per request the server
records the latency from arrival to results in host memory.

The admission and batching policy (:class:`Admission`) is plain Python and
is tested without a GPU.
"""

from __future__ import annotations

import ctypes
import gc
import time
from collections import deque
from dataclasses import dataclass, field
from functools import cached_property
from typing import Any

import numpy as np

from . import _lib
from .coding import LDPCCode, MinSum, _require_leading_info, _rule_args
from .mapping import Constellation

# Largest piece of one request's symbols a gather block copies (so one big
# request spreads over many blocks).
_CHUNK = 1 << 20


@dataclass
class Request:
    """Frames of one code on one constellation at one Es/N0."""

    rid: int
    code: str
    order: int
    symbols: Any  # (F, S) complex64: a pinned host tensor (read in place) or a CUDA tensor
    noise_var: float
    arrival: float = 0.0  # seconds from the stream's start
    # filled by the server
    admitted: float = float("nan")
    done: float = float("nan")
    bits: Any = None
    llrs: Any = None
    valid: Any = None
    iterations: Any = None

    @cached_property
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


class OutputArena:
    """A ring of pinned host memory the decoder writes results into.

    ``alloc`` hands out 256-byte aligned regions in order, wrapping at the
    end; a region still being written by a batch in flight is never handed
    out again (``busy(lo, hi)`` reports such regions, and the caller waits
    for them).
    """

    def __init__(self, nbytes: int):
        import torch

        self.buf = torch.empty(int(nbytes), dtype=torch.uint8, pin_memory=True)
        self.np = self.buf.numpy()
        self.np[:: 1 << 12] = 0  # touch every page once before serving
        self.base = self.buf.data_ptr()
        self.size = int(nbytes)
        self.head = 0

    def alloc(self, nbytes: int, busy) -> int:
        n = (int(nbytes) + 255) // 256 * 256
        if n > self.size:
            raise MemoryError(f"a batch's results ({n} bytes) exceed the {self.size}-byte output arena")
        if self.head + n > self.size:
            self.head = 0
        off = self.head
        busy(off, off + n)  # waits for batches still writing there
        self.head = off + n
        return off


class _Slot:
    """One batch slot: device buffers, pinned staging and a stream."""

    def __init__(self, server: Server, caps: dict[str, int], sym_bytes: int, max_segments: int):
        torch = server.torch
        dev = server.device
        self.stream = torch.cuda.Stream(dev)
        # The short codes' launch, on a higher-priority stream (see Server).
        self.stream_hi = torch.cuda.Stream(dev, priority=-1) if server.split else None
        self.gathered = torch.cuda.Event()
        self.hi_done = torch.cuda.Event()
        self.caps = caps
        total = sum(caps.values())
        self.sym_dev = torch.empty(sym_bytes // 8, dtype=torch.complex64, device=dev)
        self.s2_dev = torch.empty(total, dtype=torch.float32, device=dev)
        self.s2_host = torch.empty(total, dtype=torch.float32, pin_memory=True)
        self.s2_np = self.s2_host.numpy()
        self.segs = torch.empty(max_segments * 3, dtype=torch.int64, pin_memory=True)
        self.segs_np = self.segs.numpy().reshape(max_segments, 3)
        self.max_segments = max_segments
        self.llr = {}
        for name, cap in caps.items():
            self.llr[name] = torch.empty((cap, server.codes[name].n), dtype=torch.float32, device=dev)
        def workspace(entries):
            arr = server._batch_array(entries, self, {})
            need = ctypes.c_size_t(0)
            _lib.check(_lib.lib().ck_ldpc_mixed_workspace_size(arr, len(entries), ctypes.byref(need)),
                       "server slot")  # fmt: skip
            return torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=dev)

        entries = server._sizing_entries()
        self.ws = workspace(entries)
        self.ws_hi = (workspace([e if e[0] not in server.long_codes else (e[0], e[1], 0, 0, 0, 0) for e in entries])
                      if server.split else None)  # fmt: skip
        self.bytes = (self.sym_dev.numel() * 8 + self.s2_dev.numel() * 4 + self.ws.numel()
                      + (self.ws_hi.numel() if self.ws_hi is not None else 0)
                      + sum(t.numel() * 4 for t in self.llr.values()))  # fmt: skip
        self.event = torch.cuda.Event()
        self.batch: list = []
        self.layout: list = []
        self.region: tuple[int, int] | None = None
        self.out: dict = {}
        self.waiting: list = []


class Server:
    """Demap + decode server on one CUDA device (see the module docstring).

    ``frames_per_slot`` caps each code's frames in one batch; the slots'
    device memory (``max_inflight`` of them) must fit ``hbm_budget``.
    ``output_arena_bytes`` sizes the pinned result ring (by default two
    full batches of every slot).  ``fused=False`` demaps in separate
    launches before the decoder (the same bits).  ``priority_split``
    decodes the long codes' frames of a batch in their own launch, the
    others' on a higher-priority stream (the same bits).  ``spread_long``
    gives each long frame a thread block, and so an SM, of its own, with
    two threads per row slot (the same bits).
    """

    def __init__(self, codes: dict[str, LDPCCode], method: MinSum, *, hbm_budget: int = 4 << 30,
                 max_inflight: int = 3, device: Any = None, frames_per_slot: dict | None = None,
                 orders=(4, 16, 64), output_arena_bytes: int | None = None, fused: bool = True,
                 priority_split: bool = True, spread_long: bool = False):  # fmt: skip
        import torch

        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        for code in codes.values():
            _require_leading_info(code, "Server")
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
                per_frame = (code.n // kmin) * 8 + 4 + 4 * code.n
                frames_per_slot[name] = max(1, int(share // per_frame))
        self.caps = {name: int(frames_per_slot[name]) for name in codes}
        sym_bytes = sum(cap * (codes[n].n // kmin) * 8 for n, cap in self.caps.items())
        self._sym_cap = sym_bytes // 8
        out_per_slot = sum(cap * self._out_frame_bytes(n) for n, cap in self.caps.items()) + 256 * 4 * len(codes)
        if output_arena_bytes is None:
            output_arena_bytes = 2 * max_inflight * out_per_slot
        max_segments = sum(self.caps.values()) + sym_bytes // _CHUNK + 2 * len(codes) * len(self.orders) + 8
        with torch.cuda.device(self.device):
            self._tables = {o: self._axis_structs(o) for o in self.orders}
            # The decoder demaps the frames itself (one batch entry per code
            # and constellation) when every constellation allows it and the
            # entries fit one launch; else a demap launch per (code,
            # constellation) fills the slot's LLR buffers first.
            self.fused = (fused and len(codes) * len(self.orders) <= _lib.CK_LDPC_MAX_MIXED
                          and all(t[0].k == t[1].k and 1 <= t[0].k <= 4 for t in self._tables.values()))
            # Long codes (a quarter of the heaviest frame's edges or more) and
            # the others decode in separate launches of a batch, the others on
            # a higher-priority stream: the GPU does not preempt, but it hands
            # freed SMs to pending higher-priority blocks first, so short
            # requests stop queueing behind long frames not yet started.
            heaviest = max(c.checks.size for c in codes.values())
            self.long_codes = {n for n, c in codes.items() if c.checks.size * 4 >= heaviest}
            self.split = bool(priority_split and self.fused and len(self.long_codes) < len(codes))
            self.spread_long = bool(spread_long)
            self.slots = [_Slot(self, self.caps, sym_bytes, max_segments) for _ in range(max_inflight)]
        used = sum(sl.bytes for sl in self.slots)
        if used > hbm_budget:
            raise MemoryError(f"{max_inflight} batch slots need {used} bytes, over the {hbm_budget}-byte budget")
        self.hbm_bytes = used
        self.arena = OutputArena(output_arena_bytes)
        self.admission = Admission(slots=max_inflight)
        self._free = list(self.slots)
        self._busy: list[_Slot] = []
        self.completed: list[Request] = []
        self._t0 = 0.0
        self._fit: list | None = None

    def _out_frame_bytes(self, name: str) -> int:
        code = self.codes[name]
        return 4 * code.n + code.k + 4 + 1

    def _axis_structs(self, order: int):
        return _axis_structs(self.torch, self.device, order)

    def _batch_array(self, entries: list, slot: _Slot, out: dict):
        """The mixed decode's batch arguments, one per entry ``(name, order,
        B, frame offset, symbol offset, noise offset)``: ``order`` None for
        a code's LLRs in the slot's buffer, else the decoder demaps that
        constellation's frames from the slot's symbols.  Outputs at the host
        addresses ``out[name] = (llr, bits, iters, valid)`` plus the frame
        offset, or in a scratch layout when ``out`` is empty (workspace
        sizing only)."""
        arr = (_lib.Batch * len(entries))()
        m = self.method
        for i, (name, order, B, f_off, g_sym, g_s2) in enumerate(entries):
            code = self.codes[name]
            llr_o, bits_o, it_o, ok_o = out.get(name, (1, 1, 1, 1))
            if name in out:
                llr_o, bits_o = llr_o + 4 * f_off * code.n, bits_o + f_off * code.k
                it_o, ok_o = it_o + 4 * f_off, ok_o + f_off
            arr[i] = _lib.Batch(code._plan(self.device.index).handle,
                                slot.llr[name].data_ptr() + 4 * f_off * code.n, llr_o, B, code.n,
                                *_rule_args(m),
                                int(m.max_iterations), 1 if m.early_stop else 0, it_o, ok_o, bits_o,
                                code.k)  # fmt: skip
            if self.spread_long and name in self.long_codes:
                # One frame per block, on two threads per row slot.
                arr[i].frames_per_block = 1
                arr[i].threads_per_frame = 2 * ((code._plan(self.device.index).info["lifting"] + 31) // 32 * 32)
            if order is not None:
                re, im, _ = self._tables[order]
                arr[i].symbols = slot.sym_dev.data_ptr() + 8 * g_sym
                arr[i].inv_s2 = slot.s2_dev.data_ptr() + 4 * g_s2
                arr[i].axis_re = ctypes.pointer(re)
                arr[i].axis_im = ctypes.pointer(im)
        return arr

    def _sizing_entries(self) -> list:
        """Every entry at its code's full slot capacity (workspace sizing)."""
        if self.fused:
            return [(n, o, cap, 0, 0, 0) for n, cap in self.caps.items() for o in self.orders]
        return [(n, None, cap, 0, 0, 0) for n, cap in self.caps.items()]

    def _fits(self, batch: list[Request], r: Request) -> bool:
        """Whether ``r`` fits the slot beside ``batch``.  The batch's totals
        (frames per code, symbols) are kept from the previous call while the
        caller appends each accepted request, so filling a batch costs O(1)
        per request rather than a pass over the batch."""
        st = self._fit
        if st is None or st[0] is not batch or st[1] != len(batch):
            per_code: dict[str, int] = {}
            syms = 0
            for q in batch:
                per_code[q.code] = per_code.get(q.code, 0) + q.frames
                syms += q.frames * q.symbols.shape[1]
            st = self._fit = [batch, len(batch), per_code, syms]
        frames = st[2].get(r.code, 0) + r.frames
        syms = st[3] + r.frames * r.symbols.shape[1]
        ok = frames <= self.caps[r.code] and syms <= self._sym_cap
        if ok:  # the caller appends r next
            st[1] += 1
            st[2][r.code] = frames
            st[3] = syms
        return ok

    def _wait_region(self, lo: int, hi: int) -> None:
        """Blocks until no batch in flight writes into arena bytes [lo, hi)."""
        while True:
            hit = [sl for sl in self._busy if sl.region and sl.region[0] < hi and lo < sl.region[1]]
            if not hit:
                return
            self._poll(block_on=hit[0])

    def _launch(self, batch: list[Request]) -> None:
        torch = self.torch
        slot = self._free.pop()
        now = time.perf_counter() - self._t0
        slot.batch, slot.layout = batch, []
        groups: dict[tuple[str, int], list[Request]] = {}
        for r in batch:
            r.admitted = now
            groups.setdefault((r.code, r.order), []).append(r)
        segs = slot.segs_np
        sym_base, s2_base = slot.sym_dev.data_ptr(), slot.s2_dev.data_ptr()
        nseg, sym_off, s2_off = 0, 0, 0
        counts, demaps = {}, []
        for name in self.codes:
            frame_off = 0
            for order in self.orders:
                group = groups.get((name, order))
                if not group:
                    continue
                S = group[0].symbols.shape[1]
                g_sym, g_s2, g_frame = sym_off, s2_off, frame_off
                for r in group:
                    src, nbytes = r.symbols.data_ptr(), r.frames * S * 8
                    dst = sym_base + 8 * sym_off
                    for c0 in range(0, nbytes, _CHUNK):
                        segs[nseg] = (src + c0, dst + c0, min(_CHUNK, nbytes - c0))
                        nseg += 1
                    slot.s2_np[s2_off : s2_off + r.frames] = np.float32(1.0 / max(r.noise_var, 1e-20))
                    slot.layout.append((r, name, frame_off))
                    sym_off += r.frames * S
                    s2_off += r.frames
                    frame_off += r.frames
                demaps.append((order, g_sym, S, frame_off - g_frame, g_s2, name, g_frame))
            if frame_off:
                counts[name] = frame_off
        segs[nseg] = (slot.s2_host.data_ptr(), s2_base, 4 * s2_off)
        nseg += 1
        # Results go straight into the arena: per code (llrs, bits, iterations, valid).
        sizes = {n: B * self._out_frame_bytes(n) + 4 * 256 for n, B in counts.items()}
        off = self.arena.alloc(sum(sizes.values()), self._wait_region)
        slot.region = (off, off + sum(sizes.values()))
        out, slot.out = {}, {}
        a = self.arena.np
        for name, B in counts.items():
            code = self.codes[name]
            parts, o = [], off
            for nbytes in (4 * B * code.n, B * code.k, 4 * B, B):
                parts.append(o)
                o += (nbytes + 255) // 256 * 256
            # Iteration counts start at -2: the decoder publishes a frame by
            # writing its count (>= -1) last.
            a[parts[2] : parts[2] + 4 * B].view(np.int32)[:] = -2
            slot.out[name] = (B, parts, self._views(name, B, parts))
            out[name] = tuple(self.arena.base + p for p in (parts[0], parts[1], parts[2], parts[3]))
            off = o
        slot.waiting = [(r, name, off_r) for r, name, off_r in slot.layout]
        lib = _lib.lib()
        st = slot.stream.cuda_stream
        if self.split:
            self._launch_split(slot, nseg, demaps, out)
            return
        _lib.check(lib.ck_gather(slot.segs.data_ptr(), nseg, st), "server gather")
        # Every code (and constellation) takes part in every launch, with no
        # frames where a batch has none, so all batches run the one mixed
        # kernel compiled for this server's codes when its slots were built.
        if self.fused:
            got = {(name, order): (B, f_off, g_sym, g_s2) for order, g_sym, _, B, g_s2, name, f_off in demaps}
            entries = [(name, order, *got.get((name, order), (0, 0, 0, 0))) for name in self.codes
                       for order in self.orders]  # fmt: skip
        else:
            for order, g_sym, S, g_frames, g_s2, name, f_off in demaps:
                re, im, _ = self._tables[order]
                _lib.check(lib.ck_llr_separable_maxlog_frames(
                    sym_base + 8 * g_sym, g_frames * S, S, s2_base + 4 * g_s2, ctypes.byref(re), ctypes.byref(im),
                    slot.llr[name].data_ptr() + 4 * f_off * self.codes[name].n, st), "server demap")  # fmt: skip
            entries = [(name, None, counts.get(name, 0), 0, 0, 0) for name in self.codes]
        arr = self._batch_array(entries, slot, out)
        _lib.check(lib.ck_ldpc_decode_mixed(arr, len(entries), slot.ws.data_ptr(), slot.ws.numel(), st),
                   "server decode")  # fmt: skip
        slot.event.record(slot.stream)
        self._busy.append(slot)

    def _launch_split(self, slot: _Slot, nseg: int, demaps: list, out: dict) -> None:
        """The batch's gather and the short codes' decode on the slot's
        high-priority stream, the long codes' decode on its normal one; the
        slot's event completes when both have."""
        lib = _lib.lib()
        hi, lo = slot.stream_hi, slot.stream
        _lib.check(lib.ck_gather(slot.segs.data_ptr(), nseg, hi.cuda_stream), "server gather")
        slot.gathered.record(hi)
        got = {(name, order): (B, f_off, g_sym, g_s2) for order, g_sym, _, B, g_s2, name, f_off in demaps}
        for stream, ws, long in ((hi, slot.ws_hi, False), (lo, slot.ws, True)):
            if stream is lo:
                lo.wait_event(slot.gathered)
            entries = []
            for name in self.codes:
                for order in self.orders:
                    e = got.get((name, order), (0, 0, 0, 0))
                    entries.append((name, order, *(e if (name in self.long_codes) == long else (0, 0, 0, 0))))
            if any(e[2] for e in entries):
                arr = self._batch_array(entries, slot, out)
                _lib.check(lib.ck_ldpc_decode_mixed(arr, len(entries), ws.data_ptr(), ws.numel(), stream.cuda_stream),
                           "server decode")  # fmt: skip
        slot.hi_done.record(hi)
        lo.wait_event(slot.hi_done)
        slot.event.record(lo)
        self._busy.append(slot)

    def _views(self, name: str, B: int, parts: list) -> tuple:
        a, code = self.arena.np, self.codes[name]
        return (a[parts[0] : parts[0] + 4 * B * code.n].view(np.float32).reshape(B, code.n),
                a[parts[1] : parts[1] + B * code.k].view(np.int8).reshape(B, code.k),
                a[parts[2] : parts[2] + 4 * B].view(np.int32), a[parts[3] : parts[3] + B])  # fmt: skip

    def _deliver(self, slot: _Slot, r: Request, name: str, off: int, now: float) -> None:
        llrs, bits, iters, valid = slot.out[name][2]
        sl = slice(off, off + r.frames)
        r.bits, r.llrs, r.iterations = bits[sl], llrs[sl], iters[sl]
        r.valid = valid[sl].view(np.bool_)
        r.done = now
        self.completed.append(r)

    def _poll(self, block: bool = False, block_on: _Slot | None = None) -> None:
        """Delivers every request whose frames the decoder has published,
        and frees the slots whose batch is complete."""
        lib = _lib.lib()
        still = []
        for slot in self._busy:
            finished = slot.event.query()
            if not finished and (block or slot is block_on):
                slot.event.synchronize()
                finished = True
            now = time.perf_counter() - self._t0
            if finished:
                for r, name, off in slot.waiting:
                    self._deliver(slot, r, name, off, now)
                slot.waiting = []
                slot.batch, slot.layout, slot.region = [], [], None
                self._free.append(slot)
                self.admission.release()
                continue
            # Requests whose frames have all been published, before the batch ends.
            left = []
            for item in slot.waiting:
                r, name, off = item
                if int(slot.out[name][2][2][off : off + r.frames].min()) >= -1:
                    lib.ck_host_acquire()
                    self._deliver(slot, r, name, off, now)
                else:
                    left.append(item)
            slot.waiting = left
            still.append(slot)
        self._busy = still

    def serve(self, requests: list[Request]) -> list[Request]:
        """Run a request stream (arrival times in seconds from now) to completion."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        for r in pending:
            if not r.symbols.is_contiguous():
                r.symbols = r.symbols.contiguous()
            if not r.symbols.is_cuda and not r.symbols.is_pinned():
                # The gather reads payloads in place: they must be pinned (or on the device).
                r.symbols = r.symbols.pin_memory()
        self.completed = []
        # The cyclic garbage collector would pause the loop for tens of
        # milliseconds once many results are alive; requests create no cycles.
        gc_on = gc.isenabled()
        gc.disable()
        try:
            return self._serve(pending)
        finally:
            if gc_on:
                gc.enable()

    def _serve(self, pending: deque) -> list[Request]:
        torch = self.torch
        self._t0 = time.perf_counter()
        with torch.cuda.device(self.device):
            while pending or self.admission.pending or self._busy:
                now = time.perf_counter() - self._t0
                while pending and pending[0].arrival <= now:
                    self.admission.arrive(pending.popleft())
                if self._busy:
                    self._poll()
                batch = self.admission.next_batch(self._fits)
                if batch:
                    self._launch(batch)
                elif pending and not self.admission.pending and not self._busy:
                    wait = pending[0].arrival - (time.perf_counter() - self._t0)
                    if wait > 2e-4:
                        time.sleep(wait - 1e-4)
            self._poll(block=True)
        return self.completed


# ---------------------------------------------------------------------------
# Continuous feed
# ---------------------------------------------------------------------------

class FeedServer:
    """Demap + decode server over a continuous feed (``ck_ldpc_feed_launch``).

    Instead of a launch per admitted batch, one persistent decoder runs
    while requests arrive: each (code, constellation) is a queue whose
    frames the host publishes into a ring of descriptors in pinned host
    memory (where the frame's symbols are, where its results go), and the
    decoder's blocks take published frames as they free up, the queue whose
    oldest untaken frame was published first before the others.  A request
    is published whole the moment it arrives (``ck_ldpc_feed_publish``, one
    native call); nothing is copied (the decoder reads each frame's symbols
    from the request's pinned buffer and writes its results into a pinned
    output ring).  Each queue's iteration counts sit in one pinned array, so
    one vectorized test per queue finds the finished requests.  The decoder
    returns after ``idle_us`` with nothing published; the next request
    launches it again, and it continues where it stopped (the counts of
    frames taken stay in its workspace).  Results are bit-identical to
    :func:`commkit_gb300.decode` on the same LLRs.
    """

    def __init__(self, codes: dict[str, LDPCCode], method: MinSum, *, device: Any = None, orders=(4, 16, 64),
                 ring_frames: int = 1 << 14, output_arena_bytes: int = 1 << 30, idle_us: int = 20000,
                 policy: str = "oldest", max_inflight_frames: int = 8192):  # fmt: skip
        import torch

        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        for code in codes.values():
            _require_leading_info(code, "FeedServer")
        if not isinstance(method, MinSum):
            raise NotImplementedError("FeedServer decodes with MinSum")
        if ring_frames < 1 or ring_frames & (ring_frames - 1):
            raise ValueError(f"ring_frames must be a power of two, got {ring_frames}")
        self.codes, self.method, self.orders = codes, method, tuple(orders)
        self.queues = [(name, order) for name in codes for order in self.orders]
        if len(self.queues) > _lib.CK_LDPC_MAX_MIXED:
            raise ValueError(f"{len(self.queues)} (code, constellation) queues, at most {_lib.CK_LDPC_MAX_MIXED}")
        self._qidx = {q: i for i, q in enumerate(self.queues)}
        self.ring_frames = int(ring_frames)
        self.idle_us = int(idle_us)
        policies = {"oldest": _lib.CK_LDPC_FEED_OLDEST, "short_first": _lib.CK_LDPC_FEED_SHORT_FIRST}
        if policy not in policies:
            raise ValueError(f"policy must be one of {sorted(policies)}, got {policy!r}")
        self.policy = policy
        self._policy = policies[policy]
        # Frames published and not yet finished, at most (later arrivals wait
        # on the host in arrival order): keeps the host's poll short under
        # overload while the GPU still has every frame slot filled.
        self.max_inflight_frames = int(max_inflight_frames)
        nq = len(self.queues)
        lib = _lib.lib()
        with torch.cuda.device(self.device):
            self._tables = {o: _axis_structs(torch, self.device, o) for o in self.orders}
            if not all(t[0].k == t[1].k and 1 <= t[0].k <= 4 for t in self._tables.values()):
                raise NotImplementedError("FeedServer demaps in the decoder: square QAM of 4 to 256 points")
            self._arr = (_lib.Batch * nq)()
            rule, scale, offset = _rule_args(method)
            for i, (name, order) in enumerate(self.queues):
                code = codes[name]
                re, im, _ = self._tables[order]
                b = self._arr[i]
                b.plan = code._plan(self.device.index).handle
                b.n_in, b.rule, b.scale, b.offset = code.n, rule, scale, offset
                b.max_iterations, b.early_stop = int(method.max_iterations), 1 if method.early_stop else 0
                b.k_bits = code.k
                b.symbols = 1  # the frames' own symbols come from the ring
                b.axis_re, b.axis_im = ctypes.pointer(re), ctypes.pointer(im)
            # Pinned host memory: the descriptor rings, each queue's iteration
            # counts by ring slot, the published counts and the stop word.
            fb = ctypes.sizeof(_lib.FeedFrame)
            self._ring_buf = torch.zeros(nq * self.ring_frames * fb, dtype=torch.uint8, pin_memory=True)
            self._iters = torch.full((nq, self.ring_frames), -2, dtype=torch.int32, pin_memory=True)
            self._iters_np = self._iters.numpy()
            self._ctl = torch.zeros(64, dtype=torch.int32, pin_memory=True)
            self._ctl_np = self._ctl.numpy().view(np.uint32)
            base = self._ctl.data_ptr()
            self._published_addr = [base + 4 * i for i in range(nq)]
            self._stop_addr = base + 4 * 48
            self._ring_addr = [self._ring_buf.data_ptr() + i * self.ring_frames * fb for i in range(nq)]
            self._iters_addr = [self._iters.data_ptr() + 4 * i * self.ring_frames for i in range(nq)]
            self._rings = (_lib.FeedRing * nq)()
            for i in range(nq):
                self._rings[i] = _lib.FeedRing(self._ring_addr[i], self._published_addr[i], self.ring_frames)
            need = ctypes.c_size_t(0)
            _lib.check(lib.ck_ldpc_feed_workspace_size(self._arr, nq, ctypes.byref(need)), "FeedServer")
            self.ws = torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=self.device)
            self.stream = torch.cuda.Stream(self.device)
            self.event = torch.cuda.Event()
            _lib.check(lib.ck_ldpc_feed_reset(self.ws.data_ptr(), self.stream.cuda_stream), "FeedServer")
        self.hbm_bytes = self.ws.numel()
        self.arena = OutputArena(output_arena_bytes)
        self._pos = [0] * nq  # positions published per queue
        self._seq = 0
        self._running = False
        # Per queue, its requests in flight in publication order:
        # (request, first position, arena region, (llrs, bits, valid) views).
        self._inflight: list[list] = [[] for _ in range(nq)]
        self._count = 0
        self._frames = 0  # frames in flight
        self.completed: list[Request] = []
        self.launches = 0
        self._t0 = 0.0

    def _ensure_running(self) -> None:
        """Launches the decoder when it is not running (it returns when idle)."""
        if self._running and not self.event.query():
            return
        st = _lib.lib().ck_ldpc_feed_launch(self._arr, self._rings, len(self.queues), self._stop_addr, self.idle_us,
                                            self._policy, self.ws.data_ptr(), self.ws.numel(),
                                            self.stream.cuda_stream)  # fmt: skip
        _lib.check(st, "FeedServer launch")
        self.event.record(self.stream)
        self._running = True
        self.launches += 1

    def _wait_region(self, lo: int, hi: int) -> None:
        """Blocks until no request in flight has results in arena bytes [lo, hi)."""
        while any(f[2][0] < hi and lo < f[2][1] for q in self._inflight for f in q):
            self._ensure_running()
            self._poll()

    def _publish(self, r: Request, now: float) -> None:
        q = self._qidx[(r.code, r.order)]
        code = self.codes[r.code]
        F, n, k = r.frames, code.n, code.k
        if F > self.ring_frames:
            raise ValueError(f"request {r.rid}: {F} frames, the ring holds {self.ring_frames}")
        sizes = (4 * F * n, F * k, F)
        total = sum((b + 255) // 256 * 256 for b in sizes)
        off = self.arena.alloc(total, self._wait_region)
        parts, o = [], off
        for nbytes in sizes:
            parts.append(o)
            o += (nbytes + 255) // 256 * 256
        a = self.arena.np
        views = (a[parts[0] : parts[0] + sizes[0]].view(np.float32).reshape(F, n),
                 a[parts[1] : parts[1] + sizes[1]].view(np.int8).reshape(F, k), a[parts[2] : parts[2] + F])  # fmt: skip
        p0 = self._pos[q]
        # A ring slot is rewritten only after the frame it held has finished.
        while self._inflight[q] and p0 + F - self._inflight[q][0][1] > self.ring_frames:
            self._ensure_running()
            self._poll()
        base = self.arena.base
        st = _lib.lib().ck_ldpc_feed_publish(
            self._ring_addr[q], self.ring_frames, self._iters_addr[q], self._published_addr[q], p0 & 0xFFFFFFFF, F,
            r.symbols.data_ptr(), 8 * r.symbols.shape[1], base + parts[0], n, base + parts[1], k, base + parts[2],
            float(np.float32(1.0 / max(r.noise_var, 1e-20))), self._seq)  # fmt: skip
        _lib.check(st, "FeedServer publish")
        self._seq = (self._seq + F) & 0xFFFFFFFF
        self._pos[q] = p0 + F
        r.admitted = now
        self._inflight[q].append((r, p0, (off, off + total), views))
        self._count += 1
        self._frames += F

    # Requests of a queue tested per poll, oldest first: the decoder takes a
    # queue's frames in order, so later ones are rarely done before these.
    _POLL_WINDOW = 64

    def _poll(self) -> None:
        """Delivers the requests whose frames have all finished: per queue,
        one test of the iteration counts over the positions of its oldest
        requests in flight."""
        now = None
        mask = self.ring_frames - 1
        for q, every in enumerate(self._inflight):
            if not every:
                continue
            items = every[: self._POLL_WINDOW]
            lo = items[0][1]
            hi = items[-1][1] + items[-1][0].frames
            pos = np.arange(lo, hi) & mask
            done = self._iters_np[q][pos] >= -1
            starts = np.fromiter((it[1] - lo for it in items), dtype=np.int64, count=len(items))
            whole = np.logical_and.reduceat(done, starts)
            if not whole.any():
                continue
            _lib.lib().ck_host_acquire()
            if now is None:
                now = time.perf_counter() - self._t0
            keep = []
            for ok, item in zip(whole, items, strict=True):
                if not ok:
                    keep.append(item)
                    continue
                r, p, _, (llrs, bits, valid) = item
                r.llrs, r.bits, r.valid = llrs, bits, valid.view(np.bool_)
                r.iterations = self._iters_np[q][(p + np.arange(r.frames)) & mask].copy()
                r.done = now
                self.completed.append(r)
                self._count -= 1
                self._frames -= r.frames
            self._inflight[q] = keep + every[self._POLL_WINDOW :]

    def serve(self, requests: list[Request]) -> list[Request]:
        """Run a request stream (arrival times in seconds from now) to completion."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        for r in pending:
            if r.order not in self.orders or r.code not in self.codes:
                raise ValueError(f"request {r.rid}: no queue for code {r.code} on {r.order}-QAM")
            if not r.symbols.is_contiguous():
                r.symbols = r.symbols.contiguous()
            if not r.symbols.is_cuda and not r.symbols.is_pinned():
                r.symbols = r.symbols.pin_memory()  # read in place by the decoder
        self.completed = []
        gc_on = gc.isenabled()
        gc.disable()
        try:
            self._t0 = time.perf_counter()
            while pending or self._count:
                now = time.perf_counter() - self._t0
                while (pending and pending[0].arrival <= now
                       and (self._frames == 0 or self._frames + pending[0].frames <= self.max_inflight_frames)):
                    self._publish(pending.popleft(), now)
                if self._count:
                    self._ensure_running()
                    self._poll()
                elif pending:
                    wait = pending[0].arrival - (time.perf_counter() - self._t0)
                    if wait > 2e-4:
                        time.sleep(wait - 1e-4)
        finally:
            if gc_on:
                gc.enable()
        return self.completed

    def close(self) -> None:
        """Asks the decoder to return now and waits for it."""
        _lib.lib().ck_host_publish(self._stop_addr, 1)
        self.event.synchronize()
        _lib.lib().ck_host_publish(self._stop_addr, 0)
        self._running = False


def _axis_structs(torch, device, order: int):
    """The max-log axis structs of square QAM ``order`` on ``device``, and
    the device tables they point into (kept alive with them)."""
    from . import _device
    from .mapping import _axis_struct, device_tables

    like = _device.wrap(torch.empty(1, device=device))
    tabs = device_tables(Constellation.qam(order), "maxlog", like)
    half = len(tabs) // 2
    return (_axis_struct(tabs[:half], "maxlog"), _axis_struct(tabs[half:], "maxlog"), tabs)


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
