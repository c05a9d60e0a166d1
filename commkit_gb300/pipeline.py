"""Device-resident receiver pipelines: demap + decode with no per-step allocation.

:class:`MixedReceiver` holds, per code, the symbol buffer, the per-frame
``1/sigma^2``, the LLRs, the decoder outputs and one shared workspace.  A
step demaps every code's frames (``compute_llr_frames``) and decodes all of
them in ONE launch of the mixed-code persistent kernel (``decode_mixed``).
Nothing is allocated or copied inside a step, so :meth:`capture` records it
once as a CUDA graph and :meth:`run` replays it: one graph launch per batch
of mixed traffic.

The decoder takes each code's frames noisiest first (``lpt``, the
longest-processing-time-first rule: low-SNR frames run the most
iterations), so the persistent launch does not end on a tail of 50-iteration
frames; results are the same in any order.

With ``host_io=True`` the symbol buffers and the outputs are pinned host
memory instead (GB300's Grace memory is coherent with the GPU over
NVLink-C2C, with one address on both sides): the demapper reads the
received symbols where the host put them and the decoder writes each
frame's results straight into host memory, so a step needs no copy in
either direction.  The LLRs, the noise scales and the message state stay in
HBM.

With ``fused=True`` (the default) the slots whose demapping is the
closed-form max-log of a square separable constellation are demapped by the
decoder itself as it loads each frame (``ck_ldpc_batch.symbols``): a step is
then one launch, the channel LLRs never go through device memory, and with
``host_io`` the symbol reads from host memory overlap the decoding of other
frames.  The LLRs are the same bits as the demapper kernel's.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _device, _lib
from .coding import DecodeResult, LDPCCode, MinSum, _require_leading_info, _rule_args, decode_mixed
from .mapping import Constellation, _axis_struct, _table_kind, compute_llr_frames, device_tables, inv_s2_frames


@dataclass
class CodeSlot:
    """One code's frames in a :class:`MixedReceiver`."""

    code: LDPCCode
    constellation: Constellation
    frames: int
    method: MinSum
    demap: str = "maxlog"


class MixedReceiver:
    """Demap + mixed-code decode of fixed-size batches on one CUDA device."""

    def __init__(self, slots: list[CodeSlot], device: Any = None, host_io: bool = False, lpt: bool = True,
                 fused: bool = True):  # fmt: skip
        import torch

        if not slots or len(slots) > 4:
            raise ValueError("MixedReceiver: 1 to 4 code slots")
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.slots = slots
        self.host_io = bool(host_io)
        io = {"pin_memory": True} if self.host_io else {"device": self.device}
        self.sym, self.s2, self.llr, self.outputs, self.order = [], [], [], [], []
        self.lpt = bool(lpt)
        # Per slot: the (re, im) axis structs of a fused demap, or None.
        self._fused: list = []
        for s in slots:
            k = s.constellation.bits_per_symbol
            _require_leading_info(s.code, "MixedReceiver")
            if s.code.n % k:
                raise ValueError(f"n = {s.code.n} is not a multiple of {k} bits per symbol")
            S = s.code.n // k
            self.sym.append(torch.zeros((s.frames, S), dtype=torch.complex64, **io))
            self.s2.append(torch.ones((s.frames,), dtype=torch.float32, device=self.device))
            self.order.append(torch.arange(s.frames, dtype=torch.int32, device=self.device))
            self.llr.append(torch.empty((s.frames, s.code.n), dtype=torch.float32, device=self.device))
            self._fused.append(self._fusable(s) if fused else None)
            self.outputs.append((
                torch.empty((s.frames, s.code.n), dtype=torch.float32, **io),
                torch.empty((s.frames, s.code.k), dtype=torch.int8, **io),
                torch.empty((s.frames,), dtype=torch.int32, **io),
                torch.empty((s.frames,), dtype=torch.uint8, **io),
            ))  # fmt: skip
        self.workspace = torch.empty(max(self._workspace_bytes(), 256), dtype=torch.uint8, device=self.device)
        self.graph = None

    def _fusable(self, s: CodeSlot):
        """The axis structs for demapping slot ``s`` inside the decoder, or
        None where the demapper kernel runs first (level metrics, exact
        LLRs, non-separable or non-square constellations)."""
        if s.demap != "maxlog" or _table_kind(s.constellation, s.demap) != "maxlog":
            return None
        like = _device.wrap(self.llr[0] if self.llr else self.torch.empty(1, device=self.device))
        tabs = device_tables(s.constellation, "maxlog", like)
        if len(tabs) != 10:  # two axes of five tables each
            return None
        half = len(tabs) // 2
        re, im = _axis_struct(tabs[:half], "maxlog"), _axis_struct(tabs[half:], "maxlog")
        if re.k != im.k or not 1 <= re.k <= 4:
            return None
        return (re, im, tabs)

    @property
    def fused(self) -> list[bool]:
        """Per slot, whether the decoder demaps it."""
        return [f is not None for f in self._fused]

    def _batches(self) -> Any:
        arr = (_lib.Batch * len(self.slots))()
        for i, s in enumerate(self.slots):
            plan = s.code._plan(self.device.index)
            out = self.outputs[i]
            arr[i] = _lib.Batch(plan.handle, self.llr[i].data_ptr(), out[0].data_ptr(), s.frames, s.code.n,
                                *_rule_args(s.method),
                                int(s.method.max_iterations), 1 if s.method.early_stop else 0,
                                out[2].data_ptr(), out[3].data_ptr(), out[1].data_ptr(), s.code.k,
                                self.order[i].data_ptr())  # fmt: skip
            f = self._fused[i] if i < len(self._fused) else None
            if f is not None:
                arr[i].symbols = self.sym[i].data_ptr()
                arr[i].inv_s2 = self.s2[i].data_ptr()
                arr[i].axis_re = ctypes.pointer(f[0])
                arr[i].axis_im = ctypes.pointer(f[1])
        return arr

    def _workspace_bytes(self) -> int:
        need = ctypes.c_size_t(0)
        with self.torch.cuda.device(self.device):
            _lib.check(_lib.lib().ck_ldpc_mixed_workspace_size(self._batches(), len(self.slots),
                                                              ctypes.byref(need)), "MixedReceiver")  # fmt: skip
        return int(need.value)

    def load(self, symbols: list, noise_var: list) -> None:
        """Stage one batch: per slot ``(frames, S)`` complex64 symbols (host
        or device) and per-frame noise variances (host).  With ``host_io``
        the symbols go into the pinned host buffers, after the device has
        finished the steps queued before (which may still read them)."""
        if self.host_io:
            self.torch.cuda.current_stream(self.device).synchronize()
        for i, (x, nv) in enumerate(zip(symbols, noise_var, strict=True)):
            t = x if isinstance(x, self.torch.Tensor) else self.torch.from_numpy(np.ascontiguousarray(x))
            self.sym[i].copy_(t, non_blocking=True)
            s2 = inv_s2_frames(nv)
            self.s2[i].copy_(self.torch.from_numpy(s2), non_blocking=False)
            if self.lpt:
                # Longest expected first: the noisiest frames (the smallest
                # 1/sigma^2) tend to run the most iterations, so the decoder
                # takes them first and the launch ends on short frames.
                order = np.argsort(s2, kind="stable").astype(np.int32)
                self.order[i].copy_(self.torch.from_numpy(order), non_blocking=False)

    def step(self) -> None:
        """Demap every slot and decode them all in one mixed launch (no
        allocation); fused slots are demapped by the decoder."""
        if not self.host_io and not any(self.fused):
            for i, s in enumerate(self.slots):
                compute_llr_frames(self.sym[i], constellation=s.constellation, method=s.demap,
                                   inv_s2=self.s2[i], out=self.llr[i])  # fmt: skip
            decode_mixed([(self.llr[i], s.code, s.method) for i, s in enumerate(self.slots)],
                         workspace=self.workspace, outputs=self.outputs)  # fmt: skip
            return
        # The kernels through the C ABI (pinned host addresses with host_io).
        lib = _lib.lib()
        like = _device.wrap(self.llr[0])
        st = _device.stream_of(like)
        with _device.on_device(like):
            for i, s in enumerate(self.slots):
                if self._fused[i] is not None:
                    continue
                F, S = self.sym[i].shape
                kind = _table_kind(s.constellation, s.demap)
                tabs = device_tables(s.constellation, kind, like)
                exact = 1 if s.demap == "exact" else 0
                x, s2, out = self.sym[i].data_ptr(), self.s2[i].data_ptr(), self.llr[i].data_ptr()
                if kind == "points":
                    st_ = lib.ck_llr_points_frames(x, F * S, S, s2, tabs[0].data_ptr(), tabs[1].data_ptr(),
                                                   tabs[2].data_ptr(), s.constellation.order,
                                                   s.constellation.bits_per_symbol, exact, out, st)  # fmt: skip
                else:
                    half = len(tabs) // 2
                    re, im = _axis_struct(tabs[:half], kind), _axis_struct(tabs[half:], kind)
                    if kind == "maxlog":
                        st_ = lib.ck_llr_separable_maxlog_frames(x, F * S, S, s2, ctypes.byref(re),
                                                                 ctypes.byref(im), out, st)  # fmt: skip
                    else:
                        st_ = lib.ck_llr_separable_frames(x, F * S, S, s2, ctypes.byref(re), ctypes.byref(im),
                                                          exact, out, st)  # fmt: skip
                _lib.check(st_, "MixedReceiver demap")
            arr = self._batches()
            _lib.check(lib.ck_ldpc_decode_mixed(arr, len(self.slots), self.workspace.data_ptr(),
                                                self.workspace.numel(), st), "MixedReceiver decode")  # fmt: skip

    def capture(self, warmup: int = 2) -> None:
        """Record :meth:`step` as a CUDA graph (after ``warmup`` eager steps)."""
        torch = self.torch
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self.step()
        torch.cuda.current_stream(self.device).wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.step()

    def run(self) -> None:
        """One step: replay the captured graph, or run eagerly if none."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self.step()

    def results(self) -> list[DecodeResult]:
        """Each slot's result of the last step (device tensors, or pinned host
        tensors with ``host_io``; synchronize the stream before reading them)."""
        torch = self.torch
        return [DecodeResult(bits=o[1], llrs=o[0], valid=o[3].view(torch.bool), iterations=o[2], checked=True)
                for o in self.outputs]  # fmt: skip
