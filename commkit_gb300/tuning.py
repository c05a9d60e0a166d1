"""Autotuner of the decoder's launch shape, with an on-disk cache.

Every launch shape gives bit-identical results, so picking one is purely a
speed question.  :func:`tune` times the candidates for one code on the
current GPU: threads per frame (divisors and multiples of the lifting
rounded up to whole warps), frames per block, and where the check-message
state lives.  It stores the fastest in a JSON cache keyed by the GPU's name
and a digest of the code's schedule.  :func:`apply_cached` (called when a
plan is created) sets a cached shape on the plan, so tuned codes decode with
their best shape from then on.

The timing batch is what a receiver meets: frames in the code's waterfall
region, decoded with early stop, so iteration counts are as uneven as in
service and the persistent queue's balancing is part of what is timed.  By
default it is the all-zero codeword under consistent Gaussian LLRs (mean mu,
variance 2 mu, the LLRs of BPSK over AWGN), with mu found by bisection where
half the frames fail to decode; a caller may pass its own batch instead.

Cache file: ``$COMMKIT_GB300_TUNING`` or ``~/.cache/commkit_gb300/tuning.json``.
"""

from __future__ import annotations

import hashlib
import json
import os
import threading
from pathlib import Path
from typing import Any

import numpy as np

from . import _lib

_lock = threading.Lock()


def cache_path() -> Path:
    env = os.environ.get("COMMKIT_GB300_TUNING")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "commkit_gb300" / "tuning.json"


def code_key(code: Any, device_name: str) -> str:
    row_ptr, cols, layer_ptr = code._schedule
    h = hashlib.sha1()
    for a in (row_ptr, cols, layer_ptr):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    h.update(str(code.num_variables).encode())
    return f"{device_name}|{h.hexdigest()}"


def _load() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store(entries: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(f".{os.getpid()}.tmp")
        tmp.write_text(json.dumps(entries, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home is not an error: the shape just is not remembered


def _device_name(device: int) -> str:
    import torch

    return torch.cuda.get_device_name(device)


def apply_cached(code: Any, plan: Any, device: int) -> bool:
    """Set the cached shape of ``code`` on ``plan``; False if none is cached."""
    try:
        key = code_key(code, _device_name(device))
    except Exception:
        return False
    with _lock:
        entry = _load().get(key)
    if not entry:
        return False
    try:
        plan.set_launch(entry["threads_per_frame"], entry["frames_per_block"], entry["placement"])
    except ValueError:
        return False
    return True


def candidates(plan_info: dict) -> list[tuple[int, int, int]]:
    """(threads per frame, frames per block, placement) shapes to try."""
    shapes = set()
    if plan_info["quasi_cyclic"]:
        zp = (plan_info["lifting"] + 31) // 32 * 32
        ts = {t for t in (zp // d for d in (1, 2, 3, 4, 6, 8, 12)) if t >= 32 and t % 32 == 0 and zp % t == 0}
        ts |= {zp * m for m in (1, 2) if zp * m <= 768}
    else:
        ts = {32, 64, 128, 256, 512}
    for t in sorted(ts):
        for g in (0, 1, 2, 4, 8, 12):
            for place in (_lib.CK_LDPC_PLACE_SHARED, _lib.CK_LDPC_PLACE_GLOBAL):
                shapes.add((t, g, place))
            # One message per edge: the code-specialised kernel with one
            # thread per row slot (other shapes would run the records).
            if plan_info["quasi_cyclic"] and t == zp:
                shapes.add((t, g, _lib.CK_LDPC_PLACE_EDGES))
    return sorted(shapes)


def waterfall_llrs(code: Any, frames: int, *, device: int = 0, iterations: int = 50, seed: int = 0):
    """``frames`` LLR frames of the all-zero codeword in ``code``'s waterfall
    region: consistent Gaussian LLRs ``mu + sqrt(2 mu) N(0, 1)`` with ``mu``
    bisected (on a smaller batch, min-sum with early stop) to where about half
    the frames fail.  Returns ``(llrs (frames, n) float32 on the device, mu)``."""
    import torch

    from .coding import MinSum, decode

    dev = torch.device("cuda", device)
    method = MinSum(max_iterations=iterations)
    probe = max(64, min(frames, 512))
    noise = np.random.default_rng(seed).standard_normal((probe, code.n))

    def fer(mu: float) -> float:
        llr = torch.from_numpy((mu + np.sqrt(2.0 * mu) * noise).astype(np.float32)).to(dev)
        return float((~decode(llr, code=code, method=method).valid).float().mean())

    lo, hi = 0.25, 1.0
    while fer(hi) > 0.5 and hi < 1024.0:
        lo, hi = hi, 2.0 * hi
    for _ in range(7):
        mid = 0.5 * (lo + hi)
        if fer(mid) > 0.5:
            lo = mid
        else:
            hi = mid
    mu = 0.5 * (lo + hi)
    rng = np.random.default_rng(seed + 1)
    llr = (mu + np.sqrt(2.0 * mu) * rng.standard_normal((frames, code.n))).astype(np.float32)
    return torch.from_numpy(llr).to(dev), mu


def tune(code: Any, *, device: int = 0, frames: int | None = None, iterations: int = 50,
         reps: int = 3, store: bool = True, llrs: Any = None) -> dict:  # fmt: skip
    """Time the candidate shapes of ``code`` on ``device``; returns the best
    ``{"threads_per_frame", "frames_per_block", "placement", "ms", "edge_updates_per_s"}``
    (stored in the cache when ``store``) and leaves it set on the plan.
    ``llrs``: the timing batch ``(frames, n)`` on the device, else
    :func:`waterfall_llrs`; decoded with min-sum, ``iterations`` at most,
    early stop."""
    import torch

    from .coding import MinSum, decode

    dev = torch.device("cuda", device)
    plan = code._plan(device)
    info = plan.info
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    if llrs is None:
        if frames is None:
            frames = int(max(sms * 4, min(2048, (1 << 27) // max(1, code.num_variables))))
        plan.set_launch(0, 0, 0)
        llr, _ = waterfall_llrs(code, frames, device=device, iterations=iterations)
    else:
        llr = llrs.reshape(-1, code.n)
        frames = int(llr.shape[0])
    method = MinSum(max_iterations=iterations, early_stop=True)
    ws = None
    results = []
    for t, g, place in candidates(info):
        try:
            plan.set_launch(t, g, place)
            need = plan.workspace_size(frames)
        except ValueError:
            continue
        if ws is None or ws.numel() < need:
            ws = torch.empty(max(need, 256), dtype=torch.uint8, device=dev)
        decode(llr, code=code, method=method, workspace=ws)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            decode(llr, code=code, method=method, workspace=ws)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        its = int(decode(llr, code=code, method=method, workspace=ws).iterations.sum())
        results.append((ms, t, g, place, its))
    if not results:
        plan.set_launch(0, 0, 0)
        raise RuntimeError("tune(): no launch shape fits this code")
    ms, t, g, place, its = min(results)
    best = {
        "threads_per_frame": t, "frames_per_block": g, "placement": place, "ms": ms,
        "edge_updates_per_s": its * info["num_edges"] / (ms * 1e-3),
        "tried": len(results), "batch": {"frames": frames, "max_iterations": iterations, "early_stop": True,
                                        "mean_iterations": its / frames},
    }  # fmt: skip
    plan.set_launch(t, g, place)
    if store:
        with _lock:
            entries = _load()
            entries[code_key(code, _device_name(device))] = best
            _store(entries)
    return best
