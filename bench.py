"""Benchmark of the receiver back end: decoded info Gb/s at bit-identical FER.

``python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]``

Default workload: the mixed-code batch (8192 frames of codes A/B/C 60/30/10,
QPSK / 16-QAM / 16-QAM, each frame at an Eb/N0 within +-1 dB of its code's
waterfall, so iteration counts run from 2 to 50).  One step = demap every
frame and decode them all in one launch of the mixed-code persistent kernel,
replayed from a captured CUDA graph.  Inputs are seeded synthetic data
(``commkit_gb300.workloads``), drawn on the host and copied to HBM.

The line reports:
* ``value``: decoded info bits per second over the K timed steps, inputs
  resident in HBM (CUDA events on the launching stream, a barrier and a
  synchronize on both sides, max over ranks);
* ``plain``: the same frames through the public API, one ``compute_llr_frames``
  and one ``decode`` call per code, and ``batched_over_plain``;
* ``e2e``: the batched form from pinned host memory: per step the symbols
  go host -> device and every result (bits, a-posteriori LLRs, valid,
  iterations) comes back;
* ``roofline``: the decoder kernel (the dominant one) timed alone against
  its on-chip bound, shared memory (8 B of posterior traffic per edge
  update, against SMs x 128 B/clk), with the algorithmic HBM bytes against
  the measured copy bandwidth under ``hbm`` and the kernel's DRAM traffic
  from an ncu capture in ``traffic``;
* ``parity``: frames re-decoded by the CPU oracle, bit for bit;
* ``cpu_baseline``: the oracle (a C restatement of the reference's Numba
  loops, OpenMP over frames) on a bounded sample, all host threads;
* ``configs``: the other measured configurations on the same box (code C
  alone, code A alone, the demapper at 2^22 symbols, and the served request
  stream with p50/p99/p99.9 latency against load).

``--impl reference`` times the reference's CPU implementation of the path
(the oracle port: neither Numba nor CuPy is available where this runs) on
the same workload and metric with all host threads, one bounded sample per
step.  Under torchrun only rank 0 runs it.
"""

from __future__ import annotations

import argparse
import json
import os
import select
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SEED = 1
# Input/output sets a demapper leg cycles through, so that no timed launch
# finds its inputs in L2.
ROTATE = 4
METRIC = "decoded info Gb/s at bit-identical FER"
UNIT = "Gb/s"
# The measured configurations.
WORKLOADS = {
    "mixed": dict(frames=8192, max_it=50,
                  desc="mixed batch of 8192 frames: codes A/B/C 60/30/10 (QPSK, 16-QAM, 16-QAM, max-log), "
                       "per-frame Eb/N0 within +-1 dB of each code's waterfall, MinSum 50 it"),
    "C": dict(code="C", frames=4096, order=16, method="maxlog", ebn0=1.0, max_it=50,
              desc="code C (46x68 base, Z=384, N=26112, K=8448), 4096 frames, 16-QAM max-log, "
                   "Eb/N0 1.0 dB, MinSum 50 it"),
    "A": dict(code="A", frames=1024, order=4, method="exact", ebn0=2.5, max_it=20,
              desc="code A (12x24 base, Z=54, N=1296, K=648), 1024 frames, QPSK exact LLRs, "
                   "Eb/N0 2.5 dB, MinSum 20 it"),
    "demapper": dict(desc="separable demapper: 2^22 symbols, 1024 frames x 4096, per-frame Es/N0 U[8,20] dB, "
                          "16- and 64-QAM, max-log and exact"),
    "mpoint": dict(desc="M-point demapper: 16-PSK, 128-cross-QAM, 8-QAM at 2^22 symbols, max-log and exact"),
    "montecarlo": dict(desc="error_rate_curve (device Monte-Carlo loop) of codes A and C around the waterfall"),
    "dvbs2": dict(frames=64, max_it=50,
                  desc="the reference's LDPC benchmark: DVB-S2 normal frame rate 1/2 (N=64800, K=32400), "
                       "64 QPSK codewords at Es/N0 1.5 dB, one decode() call, MinSum() and SumProduct() defaults"),
    "served": dict(max_it=50,
                   desc="served stream: Poisson arrivals of 1-256 frames (log-uniform), codes A/B/C 50/35/15 "
                        "on QPSK/16-QAM/64-QAM, Es/N0 near each waterfall, MinSum 50 it, 4 GiB admission "
                        "budget over 12 batch slots, load 10-100% of measured saturation, each level three "
                        "independent 1 s streams (the median of their percentiles)"),
}  # fmt: skip


# DRAM traffic of the mixed decoder (the code-specialised kernel, codes A and B with one message
# per edge), dram__bytes_read.sum + dram__bytes_write.sum from one ncu capture (--set full) of a
# 2048-frame batch of the same mix on GB300: 20.16 + 24.91 MB.  It grows with the frames, so a
# launch's traffic is scaled by its frame count.
MIXED_DRAM_BYTES_PER_FRAME = (20.283648e6 + 23.402752e6) / 2048
MIXED_TRAFFIC_NOTE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a 2048-frame launch of the same mix "
                      "(fused demapping, codes longest first), scaled by frames (43.7 MB / 2048 frames)")


def parse() -> argparse.Namespace:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="mixed")
    ap.add_argument("--frames", type=int, default=0, help="override the workload's frame count")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="only the selected workload")
    args = ap.parse_args()
    args.w = WORKLOADS[args.workload]
    if args.frames <= 0:
        args.frames = args.w.get("frames", 0)
    return args


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0)),
                "source": "measured"}  # fmt: skip
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "fallback"}


class Clocks:
    """nvidia-smi sampling during a timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")  # fmt: skip

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.window = "the timed region"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)  # fmt: skip
        except OSError:
            self.proc = None
            return self
        # Start the timed region only once sampling runs (nvidia-smi takes a
        # while to start); that first sample, taken before it, is dropped.
        ready, _, _ = select.select([self.proc.stdout], [], [], 10.0)
        if ready:
            self.proc.stdout.readline()
        return self

    def _drain(self) -> None:
        while self.proc is not None and select.select([self.proc.stdout], [], [], 0.0)[0]:
            line = self.proc.stdout.readline()
            if not line:
                return
            self.lines.append(line)

    def keep_busy(self, step, sync, samples: int = 3, limit_s: float = 2.0) -> None:
        """For a timed region shorter than the sampling interval: repeats the
        same step (untimed, synchronised after each) right after it until
        ``samples`` readings have come in since the region began."""
        t0 = time.perf_counter()
        self.window = "the timed steps, then untimed repeats of the same step until 3 readings (50 ms apart)"
        while self.proc is not None and len(self.lines) < samples and time.perf_counter() - t0 < limit_s:
            step()
            sync()
            self._drain()

    def __exit__(self, *exc):
        if self.proc is not None:
            self._drain()
            self.proc.terminate()
            try:
                rest, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                rest, _ = self.proc.communicate()
            self.lines.extend((rest or "").splitlines())
        return False

    def summary(self) -> dict:
        rows = []
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[2:], strict=True) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "window": self.window}  # fmt: skip


class Dist:
    """Replicas over torchrun ranks: a barrier and max-over-ranks timing.

    Every rank decodes its own frames (the workload's seed includes the
    rank) and nothing is exchanged but the timings, so the whole-job rate
    is the ranks' units over the slowest rank's time.  ``backend="gloo"``
    runs the same on CPU processes (tests)."""

    def __init__(self, backend: str = "nccl"):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        import torch

        self.torch = torch
        self.cuda = backend == "nccl"
        if self.cuda:
            torch.cuda.set_device(self.local)
            self.dev = torch.device("cuda", self.local)
        else:
            self.dev = torch.device("cpu")
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group(backend, **({"device_id": self.dev} if self.cuda else {}))
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()
        if self.cuda:
            self.torch.cuda.synchronize()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def rate(self, units_per_rank: float, ms: float) -> float:
        """Whole-job units per second: every rank's units over the slowest
        rank's time (``ms``, already the maximum over ranks)."""
        return self.world * units_per_rank / (ms * 1e-3)

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


def timed(dist: Dist, fn, steps: int) -> float:
    """ms of ``steps`` calls, CUDA events on the current stream, barrier and sync both sides."""
    torch = dist.torch
    stream = torch.cuda.current_stream(dist.dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    dist.barrier()
    return dist.max(e0.elapsed_time(e1))


def timed_flushed(dist: Dist, fn, steps: int, flush) -> float:
    """ms of ``steps`` calls with the L2 flushed before each (``flush``, a
    device buffer larger than L2, is overwritten between the steps, outside
    the timed spans): the sum of per-step CUDA-event spans on the current
    stream, with a barrier and a sync on both sides."""
    torch = dist.torch
    stream = torch.cuda.current_stream(dist.dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    dist.barrier()
    for e0, e1 in ev:
        flush.zero_()
        e0.record(stream)
        fn()
        e1.record(stream)
    dist.barrier()
    return dist.max(sum(e0.elapsed_time(e1) for e0, e1 in ev))


def timed_rotating(dist: Dist, fns: list, launches: int = 20) -> float:
    """ms per launch of ``launches`` calls back to back, cycling through
    ``fns`` (the same call over distinct input and output buffers, together
    larger than L2, so that no launch finds its inputs in L2).  A device-side
    pause first lets the host queue every call, so the events time the
    kernels rather than the host; barrier and sync on both sides."""
    torch = dist.torch
    stream = torch.cuda.current_stream(dist.dev)
    for i in range(2 * len(fns)):
        fns[i % len(fns)]()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda._sleep(4_000_000)
    e0.record(stream)
    for i in range(launches):
        fns[i % len(fns)]()
    e1.record(stream)
    dist.barrier()
    return dist.max(e0.elapsed_time(e1)) / launches


def roofline(pk: dict, alg_bytes: float, edge_updates: float, launch_ms: float, sm_count: int,
             sm_mhz: float, kernel: str) -> dict:  # fmt: skip
    """The decoder's roofline.  Its bound is on chip: every edge update reads
    and writes one float of the frame's shared-memory posterior (8 B), against
    SMs x 128 B/clk x the SM clock sampled during the run; the HBM figures
    (algorithmic bytes per launch against the measured copy bandwidth) ride
    along under ``hbm``."""
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    smem_peak = sm_count * 128 * sm_mhz * 1e6 / 1e9
    smem = 8.0 * edge_updates / (launch_ms * 1e-3) / 1e9
    return {"kernel": kernel, "bound": "smem", "achieved": smem, "peak": smem_peak, "unit": "GB/s",
            "frac": smem / smem_peak, "traffic": None,
            "peak_source": f"nominal shared-memory bandwidth: {sm_count} SMs x 128 B/clk x {sm_mhz:.0f} MHz "
                           "(SM clock sampled during the run)",
            "launch_ms": launch_ms, "edge_updates": edge_updates,
            "edge_updates_per_s": edge_updates / (launch_ms * 1e-3),
            "hbm": {"achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                    "algorithmic_bytes": alg_bytes, "peak_source": pk["source"]}}  # fmt: skip


# ---------------------------------------------------------------------------
# CPU oracle samples (the reference arm and the cpu_baseline)
# ---------------------------------------------------------------------------


def _oracle_tables(spec):
    import oracle
    from commkit_gb300 import workloads as W

    checks, variables = W.lift(spec.base(), spec.z)
    m, n_var = spec.mb * spec.z, spec.nb * spec.z
    row_ptr, cols, _ = oracle.schedule(checks, variables, m, n_var)
    return row_ptr, cols, n_var, n_var - m


def oracle_step(batches, max_it: int, threads: int, method: str = "maxlog") -> tuple[float, int]:
    """The oracle's demap + decode of ``batches`` [(spec, order, symbols, noise_var, tables)]:
    (seconds, info bits).  ``noise_var`` is one value, or one per frame."""
    import oracle

    t0 = time.perf_counter()
    bits = 0
    for _spec, order, sym, nv, tables in batches:
        row_ptr, cols, n_var, k = tables
        F = sym.shape[0]
        if np.ndim(nv):
            s2 = (1.0 / np.maximum(np.asarray(nv, np.float64), 1e-20)).astype(np.float32)
            llr = oracle.llr(sym.reshape(-1), order, s2, method=method, frame_len=sym.shape[1],
                             threads=threads).reshape(F, -1)  # fmt: skip
        else:
            llr = oracle.llr(sym.reshape(-1), order, oracle.inv_s2(nv), method=method, threads=threads).reshape(F, -1)
        oracle.decode(llr, (row_ptr, cols, n_var), k=k, max_iterations=max_it, threads=threads)
        bits += F * k
    return time.perf_counter() - t0, bits


def _mixed_sample(work, fraction: float):
    from commkit_gb300 import workloads as W

    out = []
    for n, b in work.items():
        take = max(1, int(round(b.symbols.shape[0] * fraction)))
        out.append((W.CODES[n], W.MIXED_ORDERS[n], b.symbols[:take], b.noise_var[:take],
                    _oracle_tables(W.CODES[n])))  # fmt: skip
    return out


def cpu_sample(args, target_s: float):
    """A bounded sample of the workload for the oracle: about ``target_s`` of work."""
    from commkit_gb300 import workloads as W

    threads = os.cpu_count() or 1
    w = args.w
    if args.workload == "mixed":
        work = W.mixed_workload(total=args.frames)
        probe = _mixed_sample(work, 0.002)
        t, _ = oracle_step(probe, w["max_it"], threads)
        frac = min(1.0, 0.002 * target_s / max(t, 1e-3))
        sample = _mixed_sample(work, frac)
        desc = f"{frac:.2%} of each code's frames of the mixed batch ({sum(s[2].shape[0] for s in sample)} frames)"
        return sample, threads, desc
    spec = W.CODES[w["code"]]
    tables = _oracle_tables(spec)
    b = W.coded_batch(spec, threads, w["order"], w["ebn0"], seed=SEED)
    t, _ = oracle_step([(spec, w["order"], b.symbols, b.noise_var[0], tables)], w["max_it"], threads, w["method"])
    frames = int(max(threads, min(args.frames, threads * round(target_s / max(t, 1e-3)))))
    b = W.coded_batch(spec, frames, w["order"], w["ebn0"], seed=SEED)
    return [(spec, w["order"], b.symbols, b.noise_var[0], tables)], threads, f"{frames} of the {args.frames} frames"


def run_reference(args) -> None:
    """The reference arm: the CPU implementation on the host cores."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle

    oracle.build()
    sample, threads, desc = cpu_sample(args, 4.0)
    method = args.w.get("method", "maxlog")
    for _ in range(args.warmup):
        oracle_step(sample, args.w["max_it"], threads, method)
    total, bits = 0.0, 0
    for _ in range(args.steps):
        t, b = oracle_step(sample, args.w["max_it"], threads, method)
        total += t
        bits += b
    value = bits / total / 1e9
    desc = f"{desc} per step (demap + decode), {threads} threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": {"workload": args.w["desc"], "sample": desc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "oracle C restatement of commkit's Numba CPU loops (Numba and CuPy are not installed here)",
    }  # fmt: skip
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU measurements
# ---------------------------------------------------------------------------


def measure_mixed(args, dist: Dist) -> dict:
    """Config 4: the batched form (demap + one mixed-code launch from a CUDA
    graph) against the plain form (public API, one call per code)."""
    import commkit_gb300 as ck
    import oracle
    from commkit_gb300 import tuning, workloads as W
    from commkit_gb300.pipeline import CodeSlot, MixedReceiver

    torch, dev = dist.torch, dist.dev
    w = WORKLOADS["mixed"]
    frames = args.frames if args.workload == "mixed" else w["frames"]
    work = W.mixed_workload(total=frames, seed=11 + dist.rank)
    method = ck.MinSum(max_iterations=w["max_it"])
    names = list(work)
    codes = {n: ck.LDPCCode.quasi_cyclic(W.CODES[n].base(), lifting=W.CODES[n].z) for n in names}
    for n in names:  # tuned launch shapes: from the cache when this GPU has tuned the code before
        if not tuning.apply_cached(codes[n], codes[n]._plan(dev.index), dev.index):
            tuning.tune(codes[n], device=dev.index)
    consts = {n: ck.Constellation.qam(W.MIXED_ORDERS[n]) for n in names}
    rx = MixedReceiver([CodeSlot(codes[n], consts[n], work[n].symbols.shape[0], method) for n in names], dev)
    sym_host = [torch.from_numpy(work[n].symbols).pin_memory() for n in names]
    nv = [work[n].noise_var for n in names]
    rx.load(sym_host, nv)
    rx.capture()
    info_bits = sum(int(work[n].symbols.shape[0]) * codes[n].k for n in names)
    # The step's input (80 MB of symbols) fits the 126 MB L2: flush it
    # between the timed steps.
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        rx.run()
    with Clocks(dev.index) as clk:
        ms = timed_flushed(dist, rx.run, args.steps, flush)
        clk.keep_busy(lambda: (flush.zero_(), rx.run()), torch.cuda.synchronize)
    value = dist.rate(info_bits * args.steps, ms) / 1e9
    res = rx.results()

    sym_dev = [s.to(dev) for s in sym_host]

    def plain_step():
        return [ck.decode(ck.compute_llr_frames(sym_dev[i], noise_var=nv[i], constellation=consts[n]),
                          code=codes[n], method=method) for i, n in enumerate(names)]  # fmt: skip

    for _ in range(args.warmup):
        plain_step()
    plain_ms = timed_flushed(dist, plain_step, args.steps, flush)
    plain = plain_step()

    # The plain form with the reference's own calls only: its compute_llr
    # takes one noise variance, and every frame here has its own, so each
    # frame is one demapping call; then one decode call per code.
    def dropin_step():
        return [ck.decode(torch.stack([ck.compute_llr(sym_dev[i][f], noise_var=float(nv[i][f]), constellation=consts[n])
                                       for f in range(sym_dev[i].shape[0])]),
                          code=codes[n], method=method) for i, n in enumerate(names)]  # fmt: skip

    dropin_steps = max(1, min(args.steps, 3))
    dropin_step()
    dropin_ms = timed_flushed(dist, dropin_step, dropin_steps, flush)
    dropin = dropin_step()
    dropin_same = all(np.array_equal(r.llrs.cpu().numpy(), p.llrs.cpu().numpy().reshape(r.llrs.shape))
                      and np.array_equal(r.iterations.cpu().numpy(), p.iterations.cpu().numpy().reshape(-1))
                      for r, p in zip(rx.results(), dropin, strict=True))  # fmt: skip
    del dropin
    same = all(np.array_equal(r.llrs.cpu().numpy(), p.llrs.cpu().numpy().reshape(r.llrs.shape))
               and np.array_equal(r.bits.cpu().numpy(), p.bits.cpu().numpy().reshape(r.bits.shape))
               and np.array_equal(r.iterations.cpu().numpy(), p.iterations.cpu().numpy().reshape(-1))
               for r, p in zip(res, plain, strict=True))  # fmt: skip

    # The decoder launch is the whole step: it demaps each frame as it loads
    # it (every slot here is a square separable max-log constellation).
    assert all(rx.fused)
    dec_ms = ms / args.steps

    # The same receiver with the demapper kernels run first (LLRs through
    # HBM), for the record of what the fusion saves.
    rx_unf = MixedReceiver([CodeSlot(codes[n], consts[n], work[n].symbols.shape[0], method) for n in names], dev,
                           fused=False)  # fmt: skip
    rx_unf.load(sym_host, nv)
    rx_unf.capture()
    for _ in range(args.warmup):
        rx_unf.run()
    unf_ms = timed_flushed(dist, rx_unf.run, args.steps, flush)
    unf_same = all(np.array_equal(a.cpu().numpy(), b.cpu().numpy()) for r, u in zip(rx.outputs, rx_unf.outputs,
                                                                                    strict=True)
                   for a, b in zip(r, u, strict=True))  # fmt: skip
    del rx_unf

    # End to end, zero-copy: the same graph with the symbol buffers and the
    # outputs in pinned host memory.  Every step the demapper reads the
    # symbols from host memory and the decoder writes every result (LLRs,
    # bits, iterations, flags) back to it over NVLink-C2C.
    rx_io = MixedReceiver([CodeSlot(codes[n], consts[n], work[n].symbols.shape[0], method) for n in names], dev,
                          host_io=True)  # fmt: skip
    rx_io.load(sym_host, nv)
    rx_io.capture()
    for _ in range(max(1, args.warmup)):
        rx_io.run()
    e2e_ms = timed_flushed(dist, rx_io.run, args.steps, flush)
    host_same = all(np.array_equal(a.cpu().numpy(), b.numpy()) for r, h in zip(rx.outputs, rx_io.outputs, strict=True)
                    for a, b in zip(r, h, strict=True))  # fmt: skip

    # The same with explicit copies: symbols host -> device, results device -> host.
    outs = [tuple(torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in o) for o in rx.outputs]

    def copy_step():
        for i in range(len(names)):
            rx.sym[i].copy_(sym_host[i], non_blocking=True)
        rx.run()
        for o_host, o_dev in zip(outs, rx.outputs, strict=True):
            for a, b in zip(o_host, o_dev, strict=True):
                a.copy_(b, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        copy_step()
    copy_ms = timed_flushed(dist, copy_step, args.steps, flush)

    parity_ok, fer, iters, fp64 = True, {}, {}, {}
    oracle.build()
    edge_updates = 0.0
    for i, n in enumerate(names):
        F = work[n].symbols.shape[0]
        idx = np.linspace(0, F - 1, min(16, F)).astype(int)
        want = np.stack([oracle.llr(work[n].symbols[f], W.MIXED_ORDERS[n], oracle.inv_s2(work[n].noise_var[f])).reshape(-1)
                         for f in idx])  # fmt: skip
        row, col, _ = codes[n]._schedule
        ob, opost, ov, oi = oracle.decode(want, (row, col, codes[n].num_variables), k=codes[n].k,
                                          max_iterations=w["max_it"])  # fmt: skip
        r = res[i]
        # The channel LLRs of the sampled frames by the demapper kernel (the
        # fused step keeps none), then the fused step's decode of them.
        llr_dev = ck.compute_llr_frames(sym_dev[i][torch.from_numpy(idx).to(dev)], noise_var=nv[i][idx],
                                        constellation=consts[n])  # fmt: skip
        parity_ok &= (np.array_equal(llr_dev.cpu().numpy(), want)
                      and np.array_equal(r.bits.cpu().numpy()[idx], ob)
                      and np.array_equal(r.llrs.cpu().numpy()[idx], opost)
                      and np.array_equal(r.iterations.cpu().numpy()[idx], oi)
                      and np.array_equal(r.valid.cpu().numpy()[idx], ov))  # fmt: skip
        fp64[n] = decode_error_vs_fp64(r.llrs.cpu().numpy()[idx], r.iterations.cpu().numpy()[idx],
                                       r.valid.cpu().numpy()[idx], r.bits.cpu().numpy()[idx], codes[n].k, want,
                                       codes[n]._schedule, codes[n].num_variables, method.scale, method.offset,
                                       w["max_it"])  # fmt: skip
        it = r.iterations.cpu().numpy()
        edge_updates += float(it.sum()) * codes[n].checks.size
        iters[n] = [int(it.min()), round(float(it.mean()), 2), int(it.max())]
        fer[n] = float(np.mean(np.any(r.bits.cpu().numpy() != work[n].info, axis=1)))
    pk = peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    clocks = clk.summary()
    # Per frame: its symbols in (8 B each), the posterior LLRs out (4 B per
    # bit), the hard decisions, iteration count and flag.
    alg_bytes = sum(int(work[n].symbols.shape[0]) * (8 * work[n].symbols.shape[1] + 4 * codes[n].n + codes[n].k + 5)
                    for n in names)  # fmt: skip
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "frames": {n: int(work[n].symbols.shape[0]) for n in names},
                   "form": "batched: one mixed-code persistent launch per step that demaps each frame as it "
                           "loads it, CUDA-graph replay",
                   "launch_shapes": {n: codes[n]._plan(dev.index).get_launch() for n in names},
                   "l2": "flushed before every timed step (256 MB written outside the timed spans)",
                   "parallelism": f"replicas x{dist.world}"},
        "plain": {"value": dist.rate(info_bits * args.steps, plain_ms) / 1e9,
                  "ms_per_step": plain_ms / args.steps, "bit_identical_to_batched": bool(same),
                  "form": "public API: compute_llr_frames + decode, one call each per code"},
        "batched_over_plain": plain_ms / ms,
        "plain_reference_calls": {
            "value": dist.rate(info_bits * dropin_steps, dropin_ms) / 1e9,
            "ms_per_step": dropin_ms / dropin_steps, "steps": dropin_steps,
            "bit_identical_to_batched": bool(dropin_same),
            "batched_over_this": (dropin_ms / dropin_steps) / (ms / args.steps),
            "form": "the reference's drop-in calls only: compute_llr once per frame (one noise variance per call, "
                    "and every frame has its own), then decode once per code"},
        "unfused": {"value": dist.rate(info_bits * args.steps, unf_ms) / 1e9,
                    "ms_per_step": unf_ms / args.steps, "bit_identical_to_fused": bool(unf_same),
                    "form": "the demapper kernels first (LLRs through HBM), then the mixed launch"},
        "e2e": {"value": dist.rate(info_bits * args.steps, e2e_ms) / 1e9, "unit": UNIT,
                "h2d_bytes_per_step": int(sum(s.numel() * 8 for s in sym_host)),
                "d2h_bytes_per_step": int(sum(sum(t.numel() * t.element_size() for t in o) for o in outs)),
                "ms_per_step": e2e_ms / args.steps,
                "form": "MixedReceiver(host_io=True): symbols read from and results written to pinned host "
                        "memory by the kernels each step (NVLink-C2C), graph replay",
                "bit_identical_to_device": bool(host_same),
                "with_copies": {"value": dist.rate(info_bits * args.steps, copy_ms) / 1e9,
                                "ms_per_step": copy_ms / args.steps,
                                "form": "copy_ in, graph replay, copy_ out (pinned host buffers)"}},
        "gpu_launches": (1 + sum(not f for f in rx.fused)) * args.steps,
        "roofline": dict(roofline(pk, alg_bytes, edge_updates, dec_ms, sm_count, clocks.get("sm_mhz") or pk["sm_max_mhz"],
                                  "ck mixed decoder (ck_ldpc_mixed_code, code-specialised)"),
                         traffic=MIXED_DRAM_BYTES_PER_FRAME * sum(int(work[n].symbols.shape[0]) for n in names),
                         traffic_source=MIXED_TRAFFIC_NOTE),
        "decode": {"fer": fer, "iterations_min_mean_max": iters},
        "parity": {"frames_checked": 16 * len(names), "bit_exact": bool(parity_ok),
                   "decoder_vs_fp64": {"input": "the same float32 channel LLRs", "codes": fp64}},
        "clocks": clocks,
    }  # fmt: skip


def measure_single(args, dist: Dist, wname: str) -> dict:
    """Configs 3 (code C) and 1 (code A): demap + decode of one code's batch."""
    import commkit_gb300 as ck
    import oracle
    from commkit_gb300 import tuning, workloads as W

    torch, dev = dist.torch, dist.dev
    w = WORKLOADS[wname]
    frames = args.frames if args.workload == wname else w["frames"]
    spec = W.CODES[w["code"]]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    if not tuning.apply_cached(code, code._plan(dev.index), dev.index):
        tuning.tune(code, device=dev.index)
    const = ck.Constellation.qam(w["order"])
    method = ck.MinSum(max_iterations=w["max_it"])
    batch = W.coded_batch(spec, frames, w["order"], w["ebn0"], seed=SEED + dist.rank)
    nv = float(batch.noise_var[0])
    sym_host = torch.from_numpy(batch.symbols).pin_memory()
    sym = sym_host.to(dev)
    ws = torch.empty(code._plan(dev.index).workspace_size(frames), dtype=torch.uint8, device=dev)

    def step(x):
        return ck.decode(ck.compute_llr(x, noise_var=nv, constellation=const, method=w["method"]),
                         code=code, method=method, workspace=ws)  # fmt: skip

    # Code A's batch (5.3 MB of symbols) fits the L2: every timed step starts
    # from a flushed L2, as the headline's.
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        step(sym)
    ms = timed_flushed(dist, lambda: step(sym), args.steps, flush)
    res = step(sym)
    llr = ck.compute_llr(sym, noise_var=nv, constellation=const, method=w["method"])
    reps = max(3, min(args.steps, 10))
    demap_ms = timed_flushed(dist, lambda: ck.compute_llr(sym, noise_var=nv, constellation=const, method=w["method"]),
                             reps, flush) / reps  # fmt: skip
    decode_ms = timed_flushed(dist, lambda: ck.decode(llr, code=code, method=method, workspace=ws), reps, flush) / reps
    out = [torch.empty((frames, code.k), dtype=torch.int8, pin_memory=True),
           torch.empty((frames, code.n), dtype=torch.float32, pin_memory=True),
           torch.empty((frames, 1), dtype=torch.bool, pin_memory=True),
           torch.empty((frames, 1), dtype=torch.int32, pin_memory=True)]  # fmt: skip

    def e2e_step():
        r = step(sym_host.to(dev, non_blocking=True))
        for a, b in zip(out, (r.bits, r.llrs, r.valid, r.iterations), strict=True):
            a.copy_(b, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_ms = timed_flushed(dist, e2e_step, args.steps, flush)
    del flush
    iters = res.iterations.reshape(-1).cpu().numpy()
    oracle.build()
    idx = np.linspace(0, frames - 1, min(32, frames)).astype(int)
    llr_np = llr.reshape(frames, -1).cpu().numpy()[idx]
    want = oracle.llr(batch.symbols[idx].reshape(-1), w["order"], oracle.inv_s2(nv), method=w["method"]).reshape(len(idx), -1)
    llr_ok = (np.array_equal(llr_np, want) if w["method"] == "maxlog"
              else np.allclose(llr_np, want, rtol=1e-5, atol=1e-6))  # fmt: skip
    row, col, _ = code._schedule
    ob, opost, ov, oi = oracle.decode(llr_np, (row, col, code.num_variables), k=code.k, max_iterations=w["max_it"])
    bits = res.bits.reshape(frames, -1).cpu().numpy()
    post = res.llrs.reshape(frames, -1).cpu().numpy()
    valid = res.valid.reshape(-1).cpu().numpy()
    ok = (llr_ok and np.array_equal(bits[idx], ob) and np.array_equal(post[idx], opost)
          and np.array_equal(valid[idx], ov) and np.array_equal(iters[idx], oi))  # fmt: skip
    fp64 = decode_error_vs_fp64(post[idx], iters[idx], valid[idx], bits[idx], code.k, llr_np, code._schedule,
                                code.num_variables, method.scale, method.offset, w["max_it"])  # fmt: skip
    pk = peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    ksym = const.bits_per_symbol
    demap_bytes = code.n // ksym * frames * (8 + 4 * ksym)
    return {
        "workload": w["desc"], "value": dist.rate(frames * code.k * args.steps, ms) / 1e9,
        "unit": UNIT, "ms_per_step": ms / args.steps,
        "l2": "flushed before every timed step (256 MB written outside the timed spans)",
        "e2e": {"value": dist.rate(frames * code.k * args.steps, e2e_ms) / 1e9,
                "h2d_bytes_per_step": int(sym_host.numel() * 8),
                "d2h_bytes_per_step": int(sum(t.numel() * t.element_size() for t in out))},
        "launch_shape": code._plan(dev.index).get_launch(),
        "specialised": code._plan(dev.index).specialisation()[1] == 1,
        "roofline": roofline(pk, frames * (8 * code.n + code.k + 5), float(iters.sum()) * code.checks.size,
                             decode_ms, sm_count, pk["sm_max_mhz"],
                             "ck decoder (ck_ldpc_code_r*, code-specialised)"
                             if code._plan(dev.index).specialisation()[1] == 1 else "ck decoder (decode_kernel)"),
        "demapper": {"launch_ms": demap_ms, "achieved_gbs": demap_bytes / (demap_ms * 1e-3) / 1e9,
                     "frac": demap_bytes / (demap_ms * 1e-3) / 1e9 / pk["hbm_gbs"]},
        "decode": {"iterations_mean": float(iters.mean()),
                   "fer": float(np.mean(np.any(bits != batch.info, axis=1)))},
        "parity": {"frames_checked": int(len(idx)), "bit_exact": bool(ok),
                   "decoder_vs_fp64": dict(fp64, input="the same float32 channel LLRs")},
    }  # fmt: skip


def llr_fp64(x: np.ndarray, constellation, inv_s2: np.ndarray, exact: bool) -> np.ndarray:
    """The demapping formula evaluated in float64 from the kernel's float32
    inputs (symbols, points, log prior, inv_s2): metric = -|y - x|^2 inv_s2 +
    log P(x); LLR_j = log sum over points with bit j = 0 of e^metric minus
    the same over bit j = 1 (max-log: the maxima), bits MSB first
    (``commkit/mapping/_numba_llr.py:35-124``).  A checker for the error
    statement beside each demapper result, not a path that produces LLRs."""
    from commkit_gb300.mapping import host_tables

    pts, logp, lab = host_tables(constellation, "points")
    k = constellation.bits_per_symbol
    d = x.astype(np.complex128)[:, None] - pts.astype(np.complex128)[None, :]
    metric = -(d.real**2 + d.imag**2) * inv_s2.astype(np.float64)[:, None] + logp.astype(np.float64)[None, :]
    out = np.empty((x.size, k), np.float64)
    for j in range(k):
        zero = ((lab >> (k - 1 - j)) & 1) == 0
        half = []
        for sel in (zero, ~zero):
            mm = metric[:, sel]
            peak = mm.max(axis=1)
            half.append(peak + np.log(np.exp(mm - peak[:, None]).sum(axis=1)) if exact else peak)
        out[:, j] = half[0] - half[1]
    return out


def llr_error_vs_fp64(llr: np.ndarray, ref: np.ndarray) -> dict:
    """Largest absolute error, and largest relative error over entries with
    |LLR| >= 0.01 (below that, cancellation makes a ratio meaningless)."""
    err = np.abs(llr.astype(np.float64) - ref)
    big = np.abs(ref) >= 1e-2
    return {"max_abs": float(err.max()), "max_rel": float((err[big] / np.abs(ref[big])).max()) if big.any() else 0.0}


FP64_SAMPLE = 1 << 16


def decode_fp64(llr: np.ndarray, schedule, n_var: int, scale: float, offset: float, max_it: int,
                dtype=np.float64):
    """The layered min-sum decode evaluated in float64 from the decoder's
    float32 input LLRs: per row Q = APP - R, min1/min2/first argmin and the
    sign parity of Q, R' = sign * max(scale min - offset, 0) (min2 at the
    argmin), APP = Q + R', rows in the schedule's layer order, a syndrome
    test before the first iteration and after each one
    (``commkit/coding/_numba_loops.py:43-68,97-147``).  The rows of a layer
    share no variable, so a layer is one vectorised step over its rows and
    the frames.  Returns (posteriors, iterations, valid).  A checker for the
    error statement beside the decoder's results, not a decoding path;
    ``dtype=np.float32`` evaluates the same steps in the decoder's own
    precision (the CPU tests hold that to the oracle bit for bit)."""
    row_ptr, cols, layer_ptr = (np.asarray(a, np.int64) for a in schedule)
    F, n = llr.shape
    E = int(row_ptr[-1])
    layers = []  # per layer: edge ids and columns (rows x widest row), padded with a dummy edge E / column n_var
    for l in range(layer_ptr.size - 1):
        rows = np.arange(layer_ptr[l], layer_ptr[l + 1])
        deg = row_ptr[rows + 1] - row_ptr[rows]
        D = int(deg.max())
        pos = np.arange(D)[None, :]
        mask = pos < deg[:, None]
        eid = np.where(mask, row_ptr[rows][:, None] + pos, E)
        cid = np.where(mask, np.append(cols, n_var)[eid], n_var)
        layers.append((eid, cid, mask))
    app = np.zeros((F, n_var + 1), dtype)
    app[:, :n] = llr.astype(dtype)
    msg = np.zeros((F, E + 1), dtype)
    scale, offset = dtype(scale), dtype(offset)
    one = dtype(1.0)
    check_rows = np.repeat(np.arange(row_ptr.size - 1), np.diff(row_ptr))

    def satisfied(a):
        neg = (a[:, cols] < 0).astype(np.int64)
        par = np.zeros((a.shape[0], row_ptr.size - 1), np.int64)
        np.add.at(par.T, check_rows, neg.T)
        return ~np.any(par & 1, axis=1)

    iters = np.zeros(F, np.int32)
    live = ~satisfied(app)
    for _ in range(max_it):
        f = np.flatnonzero(live)
        if f.size == 0:
            break
        a, r = app[f], msg[f]
        for eid, cid, mask in layers:
            q = a[:, cid] - r[:, eid]
            mag = np.where(mask, np.abs(q), np.inf)
            order = np.argsort(mag, axis=2, kind="stable")  # the first edge holding min1 comes first
            min1 = np.take_along_axis(mag, order[..., :1], axis=2)
            min2 = np.take_along_axis(mag, order[..., 1:2], axis=2) if mag.shape[2] > 1 else np.full_like(min1, np.inf)
            neg = (q < 0) & mask
            par = np.logical_xor.reduce(neg, axis=2, keepdims=True)
            n1 = np.maximum(scale * min1 - offset, dtype(0.0))
            n2 = np.maximum(scale * min2 - offset, dtype(0.0))
            at = np.arange(mask.shape[1])[None, None, :] == order[..., :1]
            rn = np.where(at, n2, n1) * np.where(par ^ neg, -one, one)
            a[:, cid[mask]] = (q + rn)[:, mask]
            r[:, eid[mask]] = rn[:, mask]
        app[f], msg[f] = a, r
        iters[f] += 1
        live[f] = ~satisfied(a)
    return app[:, :n], iters, ~live


def decode_error_vs_fp64(post: np.ndarray, iters: np.ndarray, valid: np.ndarray, bits: np.ndarray, k: int,
                         llr: np.ndarray, schedule, n_var: int, scale: float, offset: float, max_it: int) -> dict:
    """The decoder's float32 results against ``decode_fp64`` of the same
    input LLRs, split by outcome.  Frames that converged: how many take the
    same iteration count, the same validity and the same hard decisions in
    float64, and over those with the same count the largest absolute
    posterior error and the largest relative to the frame's largest
    |posterior|.  Frames that ran every iteration without converging: how
    many keep the same hard decisions (min-sum on a frame it cannot decode
    wanders, and float32 and float64 rounding send it along different
    paths, so these are counted, not compared)."""
    p64, i64, v64 = decode_fp64(llr, schedule, n_var, scale, offset, max_it)
    valid = np.asarray(valid).astype(bool).reshape(-1)
    same_bits = np.all(bits.astype(bool) == (p64[:, :k] < 0), axis=1)
    ok = valid
    same = ok & (iters == i64) & v64
    conv = {"frames": int(ok.sum()), "same_iterations_and_valid": int(same.sum()),
            "same_bits": int((same_bits & ok).sum())}  # fmt: skip
    if same.any():
        err = np.abs(post[same].astype(np.float64) - p64[same])
        peak = np.maximum(np.abs(p64[same]).max(axis=1, keepdims=True), 1e-30)
        conv.update(max_abs=float(err.max()), max_rel_to_frame_peak=float((err / peak).max()))
    return {"converged": conv,
            "unconverged": {"frames": int((~ok).sum()), "same_bits": int((same_bits & ~ok).sum())}}


def measure_demapper(dist: Dist) -> dict:
    """Config 2: 2^22 symbols in 1024 frames of 4096, per-frame Es/N0 in
    [8, 20] dB, 16- and 64-QAM, max-log and exact, one batched launch;
    timed 20 launches back to back over four sets of symbols and outputs,
    so that no launch finds its inputs in L2."""
    import commkit_gb300 as ck
    from commkit_gb300 import workloads as W
    from commkit_gb300.mapping import inv_s2_frames

    torch, dev = dist.torch, dist.dev
    pk = peaks()
    out = {}
    for order in (16, 64):
        rx, nv = W.demapper_batch(order, frames=1024, frame_len=4096, seed=3)
        x = torch.from_numpy(rx).to(dev)
        s2 = torch.from_numpy(inv_s2_frames(nv)).to(dev)
        c = ck.Constellation.qam(order)
        # Four sets of symbols and outputs (403 / 537 MB in all, against a
        # 129 MB L2: 16-QAM's 101 MB of one launch alone would fit it).
        xs = [x] + [x.clone() for _ in range(ROTATE - 1)]
        res = [torch.empty((1024, 4096 * c.bits_per_symbol), dtype=torch.float32, device=dev) for _ in xs]
        for method in ("maxlog", "exact"):
            fns = [lambda method=method, xi=xi, ri=ri: ck.compute_llr_frames(xi, constellation=c, method=method,
                                                                             inv_s2=s2, out=ri)
                   for xi, ri in zip(xs, res, strict=True)]  # fmt: skip
            for _ in range(5):  # also brings the clocks up when this leg runs first
                for fn in fns:
                    fn()
            ms = timed_rotating(dist, fns)
            nbytes = rx.size * (8 + 4 * c.bits_per_symbol) + 1024 * 4
            k = c.bits_per_symbol
            got = res[0].reshape(-1, k)[:FP64_SAMPLE].cpu().numpy()
            ref = llr_fp64(rx.reshape(-1)[:FP64_SAMPLE], c, np.repeat(inv_s2_frames(nv), 4096)[:FP64_SAMPLE],
                           method == "exact")  # fmt: skip
            out[f"qam{order}_{method}"] = {"us": ms * 1e3, "gbs": nbytes / (ms * 1e-3) / 1e9,
                                           "frac": nbytes / (ms * 1e-3) / 1e9 / pk["hbm_gbs"],
                                           "err_vs_fp64": llr_error_vs_fp64(got, ref)}  # fmt: skip
    # Same-traffic calibration: device-to-device copies (torch copy_ of
    # contiguous buffers, cudaMemcpyAsync) with the demapper's reads and
    # writes: the 8-byte symbols copied k / 2 times into an output of 4k
    # bytes per symbol, timed the same way (L2 flushed first): what this GPU
    # sustains for that stream with no arithmetic at all, against the copy
    # peak measured on 2 GB.
    calib = {}
    srcs = [torch.view_as_real(xi).reshape(-1) for xi in xs]
    del res
    for order in (16, 64):
        reps = int(np.log2(order)) // 2
        dsts = [torch.empty((reps, srcs[0].numel()), dtype=torch.float32, device=dev) for _ in srcs]

        def copies(src, dst, reps=reps):
            for r in range(reps):
                dst[r].copy_(src)

        us = timed_rotating(dist, [lambda a=a, b=b: copies(a, b) for a, b in zip(srcs, dsts, strict=True)]) * 1e3
        nbytes = srcs[0].numel() * 4 + reps * srcs[0].numel() * 4
        calib[f"qam{order}"] = {"copies": reps, "us": us, "gbs": nbytes / (us * 1e-6) / 1e9,
                                "maxlog_kernel_over_copies": out[f"qam{order}_maxlog"]["us"] / us}  # fmt: skip
        del dsts
    return {"workload": f"2^22 symbols, 1024 frames x 4096, per-frame Es/N0 U[8,20] dB, one launch, 20 launches "
                        f"back to back over {ROTATE} sets of inputs and outputs (larger than L2 together)",
            "fp64_sample_symbols": FP64_SAMPLE, "results": out,
            "same_traffic_calibration": {"what": "k/2 device-to-device copies of the symbols into a 4k-byte-per-symbol "
                                                 "output (the demapper's reads and writes, no arithmetic), timed as the "
                                                 "kernels: 20 back to back over the same rotating buffers",
                                         "results": calib}}  # fmt: skip


def measure_mpoint(dist: Dist) -> dict:
    """The M-point demapper (constellations without per-axis factors) at
    2^22 symbols: 16-PSK and 128-cross-QAM, the reference's non-separable
    benchmark constellations (``benchmarks/bench_llr.py:38-51``, there at
    2^18 symbols), and 8-QAM; max-log and exact; 20 launches back to back
    over four copies of the symbols (and four outputs), so that no launch
    finds its inputs in L2; the calls' host work is queued ahead behind a
    device-side pause, so the events time the kernels."""
    import commkit_gb300 as ck
    from commkit_gb300.mapping import inv_s2

    torch, dev = dist.torch, dist.dev
    pk = peaks()
    out = {}
    for name, c in (("psk16", ck.Constellation.psk(16)), ("qam128_cross", ck.Constellation.qam(128)),
                    ("qam8", ck.Constellation.qam(8))):  # fmt: skip
        n = 1 << 22
        rng = np.random.default_rng(5)
        x = c.points[rng.integers(0, c.order, n)] + 0.1 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
        xd = torch.from_numpy(x.astype(np.complex64)).to(dev)
        xs = [xd] + [xd.clone() for _ in range(ROTATE - 1)]
        for method in ("maxlog", "exact"):
            # Each call allocates its output; the last ROTATE outputs stay
            # alive, so the outputs rotate over distinct buffers as well.
            kept = [None] * ROTATE

            def call(i, method=method):
                kept[i] = ck.compute_llr(xs[i], noise_var=0.05, constellation=c, method=method)

            ms = timed_rotating(dist, [lambda i=i: call(i) for i in range(ROTATE)])
            del kept
            nbytes = n * (8 + 4 * c.bits_per_symbol)
            got = ck.compute_llr(xd[:FP64_SAMPLE], noise_var=0.05, constellation=c, method=method)
            got = got.cpu().numpy().reshape(FP64_SAMPLE, -1)
            ref = llr_fp64(x[:FP64_SAMPLE].astype(np.complex64), c,
                           np.full(FP64_SAMPLE, inv_s2(0.05), np.float32), method == "exact")  # fmt: skip
            out[f"{name}_{method}"] = {"us": ms * 1e3, "gsym_per_s": n / (ms * 1e-3) / 1e9,
                                       "gbs": nbytes / (ms * 1e-3) / 1e9,
                                       "frac": nbytes / (ms * 1e-3) / 1e9 / pk["hbm_gbs"],
                                       "err_vs_fp64": llr_error_vs_fp64(got, ref)}  # fmt: skip
    return {"workload": "M-point demapping, 2^22 symbols per call (public compute_llr), 20 calls back to back "
                        f"over {ROTATE} sets of symbols and outputs (larger than L2 together)",
            "fp64_sample_symbols": FP64_SAMPLE, "results": out}


def measure_montecarlo(dist: Dist) -> dict:
    """The Monte-Carlo error-rate loop (``error_rate_curve``) of codes A and
    C at three Es/N0 points around each waterfall, a fixed number of blocks
    per point (no early end on errors): bits, encoding, mapping, noise,
    demapping, decoding and error counts all on the device, one 56-byte
    result copy per batch.  At the reference's batch (2^18 transmitted bits,
    203 / 10 blocks) and at 4096-block batches."""
    import torch

    import commkit_gb300 as ck
    from commkit_gb300 import workloads as W

    out = {}
    for name, order in (("A", 4), ("C", 16)):
        spec = W.CODES[name]
        code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
        c = ck.Constellation.qam(order)
        k = int(round(np.log2(order)))
        es0 = W.WATERFALL_DB[name] + 10 * np.log10(code.k / code.n * k)
        grid = [es0 - 0.5, es0, es0 + 0.5]
        for label, batch, blocks in (("reference_batch", None, 4096 if name == "A" else 1024),
                                     ("batch_4096", 4096, 16384 if name == "A" else 8192)):  # fmt: skip
            kw = dict(constellation=c, esn0_db=grid, method=ck.MinSum(max_iterations=50), min_block_errors=10**9,
                      max_blocks=blocks, rng=1, batch_blocks=batch)  # fmt: skip
            ck.error_rate_curve(code, **{**kw, "max_blocks": min(blocks, 512)})  # warm-up (plans, graphs)
            torch.cuda.synchronize(dist.dev)
            t = time.perf_counter()
            curve = ck.error_rate_curve(code, **kw)
            torch.cuda.synchronize(dist.dev)
            dt = time.perf_counter() - t
            nblk = int(np.sum(curve.num_blocks))
            out[f"{name}_{label}"] = {"blocks": nblk, "s": dt, "blocks_per_s": nblk / dt,
                                      "info_gbps": nblk * code.k / dt / 1e9, "fer": [float(v) for v in curve.fer],
                                      "mean_iterations": [float(v) for v in curve.mean_iterations]}  # fmt: skip
    return {"workload": "error_rate_curve of codes A (QPSK) and C (16-QAM) at the waterfall Es/N0 and +-0.5 dB, "
                        "MinSum 50 it, fixed blocks per point, wall clock of the public call", "results": out}


def measure_host_overhead(dist: Dist, batches: int = 30, per_batch: int = 100) -> dict:
    """Host time per public call: ``compute_llr`` of 4096 16-QAM symbols and
    ``decode`` of one code-A frame, each with its outputs allocated by the
    call, as a drop-in user who calls per frame runs them.  Timed over
    batches of ``per_batch`` calls with the GPU drained between batches
    (outside the timed spans), so the launch queue never fills and blocks
    the host; the median batch gives the figure.  ``sustained`` is 2000
    calls back to back, where a kernel longer than the host work sets the
    pace instead."""
    import commkit_gb300 as ck
    from commkit_gb300 import workloads as W

    torch, dev = dist.torch, dist.dev
    c = ck.Constellation.qam(16)
    x = torch.from_numpy((np.random.default_rng(3).standard_normal(8192).astype(np.float32)).view(np.complex64)).to(dev)
    code = ck.LDPCCode.quasi_cyclic(W.CODE_A.base(), lifting=W.CODE_A.z)
    llr = torch.from_numpy((2.0 + np.random.default_rng(4).standard_normal(code.n)).astype(np.float32)).to(dev)
    method = ck.MinSum(max_iterations=20)
    out, sustained = {}, {}
    for name, fn in (("compute_llr_4096_symbols", lambda: ck.compute_llr(x, noise_var=0.1, constellation=c)),
                     ("decode_1_frame_code_A", lambda: ck.decode(llr, code=code, method=method))):  # fmt: skip
        for _ in range(200):
            fn()
        torch.cuda.synchronize(dev)
        per = []
        for _ in range(batches):
            t0 = time.perf_counter()
            for _ in range(per_batch):
                fn()
            per.append((time.perf_counter() - t0) / per_batch * 1e6)
            torch.cuda.synchronize(dev)
        out[name] = float(np.median(per))
        t0 = time.perf_counter()
        for _ in range(2000):
            fn()
        sustained[name] = (time.perf_counter() - t0) / 2000 * 1e6
        torch.cuda.synchronize(dev)
    from commkit_gb300 import _lib

    return {"unit": "us per call (host)", "calls": batches * per_batch, "results": out,
            "sustained_2000_calls": sustained, "per_call_extension": _lib.calls() is not None,
            "timing": f"median of {batches} batches of {per_batch} calls, the GPU drained between batches"}  # fmt: skip


def measure_dvbs2(dist: Dist, steps: int = 10, warmup: int = 3) -> dict:
    """The reference's own LDPC benchmark (``benchmarks/bench_coding.py:37-38,
    55-56,75-86``): 64 DVB-S2 normal-frame rate-1/2 codewords over QPSK at
    Es/N0 1.5 dB, LLRs on the device, one ``decode`` call per step (outputs
    allocated by the call, as the reference's).  Its published medians on an
    RTX 4070 Ti are 15.745 ms (MinSum) and 13.982 ms (SumProduct).  The
    codewords, encoded by this package's accumulator encoder, decode
    bit-identically to the oracle; the L2 is flushed before every step."""
    import commkit_gb300 as ck
    import oracle
    from commkit_gb300.workloads import awgn, encode_accumulate, map_bits

    torch, dev = dist.torch, dist.dev
    d = np.load(ROOT / "tests" / "golden" / "dvbs2_normal.npz")
    m, N, n, k = (int(d[f"dvbs2n_{s}"]) for s in ("m", "N", "n", "k"))
    code = ck.LDPCCode(d["dvbs2n_checks"], d["dvbs2n_variables"], m, N, N - n)
    F = WORKLOADS["dvbs2"]["frames"]
    rng = np.random.default_rng(SEED + dist.rank)
    info = rng.integers(0, 2, size=(F, k), dtype=np.int8)
    nv = 10.0 ** (-1.5 / 10.0)
    sym = awgn(map_bits(encode_accumulate(d["dvbs2n_checks"], d["dvbs2n_variables"], m, k, info), 4), nv, rng)
    llr = ck.compute_llr(torch.from_numpy(sym).to(dev), noise_var=nv, constellation=ck.Constellation.qam(4))
    llr = llr.reshape(F, n)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    out = {"workload": WORKLOADS["dvbs2"]["desc"]}
    for name, method, ref_ms in (("min_sum", ck.MinSum(), 15.745), ("sum_product", ck.SumProduct(), 13.982)):
        for _ in range(warmup):
            res = ck.decode(llr, code=code, method=method)
        times = []
        for _ in range(steps):
            flush.zero_()
            times.append(timed(dist, lambda method=method: ck.decode(llr, code=code, method=method), 1))
        ms = float(np.median(times))
        iters = res.iterations.cpu().numpy().reshape(-1)
        entry = {"ms": ms, "mbps": F * k / (ms * 1e-3) / 1e6, "iterations_mean": float(iters.mean()),
                 "frames_decoded": int(res.valid.cpu().numpy().sum()), "frames": F,
                 "reference_published_ms_rtx4070ti": ref_ms}  # fmt: skip
        if name == "min_sum" and dist.rank == 0:
            row_ptr, cols, _ = code._schedule
            want = oracle.decode(llr[:4].cpu().numpy(), (row_ptr, cols, N), k=k, max_iterations=50)
            entry["parity_4_frames_bit_exact"] = bool(
                np.array_equal(res.llrs.cpu().numpy().reshape(F, -1)[:4], want[1])
                and np.array_equal(iters[:4], want[3]))  # fmt: skip
        out[name] = entry
    return out


def measure_served(args, dist: Dist) -> dict:
    """Config 5: the continuous-batching server under Poisson load."""
    import commkit_gb300 as ck
    from commkit_gb300 import workloads as W
    from commkit_gb300.serving import PayloadPool, Server, poisson_requests

    dev = dist.dev
    t_build = time.perf_counter()
    pool = PayloadPool.build({(n, o): {"A": 4096, "B": 2048, "C": 384}[n] for n in "ABC" for o in (4, 16, 64)},
                             seed=7)  # fmt: skip
    t_build = time.perf_counter() - t_build
    codes = {n: ck.LDPCCode.quasi_cyclic(W.CODES[n].base(), lifting=W.CODES[n].z) for n in "ABC"}
    slots = int(os.environ.get("CK_SERVE_SLOTS", "12"))
    # 4 GiB per 12 slots: every slot holds a full request of each code.
    server = Server(codes, ck.MinSum(max_iterations=WORKLOADS["served"]["max_it"]),
                    hbm_budget=max(4 << 30, slots * ((4 << 30) // 12)), max_inflight=slots, device=dev,
                    spread_long=os.environ.get("CK_SERVE_SPREAD", "0") == "1")  # fmt: skip
    k_of = {n: c.k for n, c in codes.items()}

    def info_bits(reqs):
        return sum(r.frames * k_of[r.code] for r in reqs)

    server.serve(poisson_requests(1e5, 0.002, pool, seed=1))  # warm-up
    # Saturation: the sustained completion rate under overload.  A first
    # backlog (everything arrived at once) gives a rough rate; then requests
    # arrive at 3x that rate for 0.5 s, and the rate is what the server
    # completes from the first arrival until the backlog has drained.
    backlog = poisson_requests(1e6, 4e-4, pool, seed=2)
    for r in backlog:
        r.arrival = 0.0
    t0 = time.perf_counter()
    server.serve(backlog)
    rough = len(backlog) / (time.perf_counter() - t0)
    over = poisson_requests(3.0 * rough, 0.5, pool, seed=3)
    t0 = time.perf_counter()
    server.serve(over)
    sat_s = time.perf_counter() - t0
    sat_rate = len(over) / sat_s
    backlog = over
    duration = float(os.environ.get("CK_SERVE_SECONDS", "1.0"))
    reps = int(os.environ.get("CK_SERVE_REPS", "3"))
    sweep = {}
    with Clocks(dev.index) as clk:
        for load in (0.1, 0.3, 0.5, 0.7, 0.9, 1.0):
            runs = []
            for rep in range(reps):
                reqs = poisson_requests(load * sat_rate, duration, pool, seed=int(load * 100) + 1000 * rep)
                t0 = time.perf_counter()
                done = server.serve(reqs)
                runs.append((done, time.perf_counter() - t0))
            sweep[f"{int(round(load * 100))}%"] = _load_level(runs, info_bits, waits=True)
    feed = {policy: measure_feed(codes, pool, sat_rate, duration, info_bits, dev, policy)
            for policy in ("oldest", "short_first")}
    return {
        "workload": WORKLOADS["served"]["desc"],
        "feed": feed,
        "saturation": {"gbps": info_bits(backlog) / sat_s / 1e9, "requests_per_s": sat_rate,
                       "requests": len(backlog), "frames": int(sum(r.frames for r in backlog)),
                       "method": "overload at 3x a backlog estimate for 0.5 s, completed / wall until drained"},
        "latency_vs_load": sweep, "p99_ms_at_70pct": sweep["70%"]["p99_ms"], "batch_slots": slots,
        "policy": {"fused": server.fused, "priority_split": server.split, "long_codes": sorted(server.long_codes),
                   "spread_long": server.spread_long},
        "pool_build_s": t_build, "clocks": clk.summary(),
    }  # fmt: skip


def _latency_summary(done, wall: float, info_bits, waits: bool = False) -> dict:
    lat = np.array([r.latency for r in done]) * 1e3
    out = {"requests": len(done), "frames": int(sum(r.frames for r in done)),
           "gbps": info_bits(done) / wall / 1e9, "p50_ms": float(np.percentile(lat, 50)),
           "p99_ms": float(np.percentile(lat, 99)), "p999_ms": float(np.percentile(lat, 99.9)),
           "max_ms": float(lat.max()),
           "p99_ms_by_code": {c: float(np.percentile([r.latency * 1e3 for r in done if r.code == c], 99))
                              for c in "ABC" if any(r.code == c for r in done)}}  # fmt: skip
    if waits:
        # Time from arrival to admission into a batch slot: the queueing part of the latency.
        out["p99_wait_ms"] = float(np.percentile([(r.admitted - r.arrival) * 1e3 for r in done], 99))
        out["p99_wait_ms_by_code"] = {c: float(np.percentile([(r.admitted - r.arrival) * 1e3 for r in done
                                                              if r.code == c], 99))
                                      for c in "ABC" if any(r.code == c for r in done)}  # fmt: skip
    return out


def _load_level(runs, info_bits, waits: bool = False) -> dict:
    """One load level measured as independent request streams (different
    seeds) served one after another: each stream's percentiles, and their
    median as the level's figure, so a single host stall of a few
    milliseconds in one stream (seen now and then on the GPU machine, cause
    unknown) shows in that stream's entry instead of deciding the level."""
    per = [_latency_summary(done, wall, info_bits, waits) for done, wall in runs]
    med = {k: float(np.median([p[k] for p in per])) for k in per[0] if isinstance(per[0][k], float)}
    med.update(requests=int(sum(p["requests"] for p in per)), frames=int(sum(p["frames"] for p in per)),
               gbps=float(sum(info_bits(d) for d, _ in runs) / sum(w for _, w in runs) / 1e9))  # fmt: skip
    for key in ("p99_ms_by_code", "p99_wait_ms_by_code"):
        if key in per[0]:
            med[key] = {c: float(np.median([p[key][c] for p in per if c in p[key]])) for c in per[0][key]}
    med["streams"] = len(per)
    med["p99_ms_each"] = [p["p99_ms"] for p in per]
    med["max_ms_each"] = [p["max_ms"] for p in per]
    return med


def measure_feed(codes, pool, sat_rate: float, duration: float, info_bits, dev, policy: str) -> dict:
    """Config 5 through the continuous feed (``serving.FeedServer``): the
    same request streams (the same seeds and rates, as fractions of the
    batched server's saturation) published into one running decoder, whose
    blocks take the oldest queue first, or the short codes' queues first."""
    import commkit_gb300 as ck
    from commkit_gb300.serving import FeedServer, poisson_requests

    server = FeedServer(codes, ck.MinSum(max_iterations=WORKLOADS["served"]["max_it"]), device=dev,
                        output_arena_bytes=2 << 30, idle_us=20000, policy=policy)  # fmt: skip
    server.serve(poisson_requests(1e5, 0.002, pool, seed=1))  # warm-up (compiles and loads the kernel)
    over = poisson_requests(3.0 * sat_rate, 0.5, pool, seed=3)
    t0 = time.perf_counter()
    done = server.serve(over)
    sat_s = time.perf_counter() - t0
    sweep = {}
    reps = int(os.environ.get("CK_SERVE_REPS", "3"))
    with Clocks(dev.index) as clk:
        for load in (0.1, 0.3, 0.5, 0.7, 0.9):
            runs = []
            for rep in range(reps):
                reqs = poisson_requests(load * sat_rate, duration, pool, seed=int(load * 100) + 1000 * rep)
                t0 = time.perf_counter()
                got = server.serve(reqs)
                runs.append((got, time.perf_counter() - t0))
            sweep[f"{int(round(load * 100))}%"] = _load_level(runs, info_bits)
    launches = server.launches
    server.close()
    return {"what": "one persistent decoder fed from pinned descriptor rings (ck_ldpc_feed_launch); loads are "
                    "fractions of the batched server's saturation",
            "saturation_gbps": info_bits(done) / sat_s / 1e9, "latency_vs_load": sweep,
            "p99_ms_at_70pct": sweep["70%"]["p99_ms"], "launches": launches, "clocks": clk.summary()}  # fmt: skip


def main() -> None:
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    dist = Dist()
    if args.workload == "mixed":
        line = measure_mixed(args, dist)
    elif args.workload == "demapper":
        dm = measure_demapper(dist)
        r = dm["results"]["qam16_maxlog"]
        line = {"metric": "demapper HBM throughput", "value": r["gbs"], "unit": "GB/s", "n_gpus": 1, "steps": 10,
                "warmup": 3, "ms_per_step": r["us"] / 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": dm["workload"]}, "demapper": dm}  # fmt: skip
    elif args.workload == "mpoint":
        mp_ = measure_mpoint(dist)
        r = mp_["results"]["qam128_cross_maxlog"]
        line = {"metric": "M-point LLR throughput", "value": r["gsym_per_s"], "unit": "Gsymbols/s", "n_gpus": 1,
                "steps": 10, "warmup": 3, "ms_per_step": r["us"] / 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": mp_["workload"]}, "mpoint": mp_}  # fmt: skip
    elif args.workload == "montecarlo":
        mc = measure_montecarlo(dist)
        r = mc["results"]["C_batch_4096"]
        line = {"metric": "Monte-Carlo decoded info Gb/s", "value": r["info_gbps"], "unit": UNIT, "n_gpus": 1,
                "steps": 1, "warmup": 1, "ms_per_step": r["s"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": mc["workload"]}, "montecarlo": mc}  # fmt: skip
    elif args.workload == "dvbs2":
        dv = measure_dvbs2(dist, args.steps, args.warmup)
        ms = dv["min_sum"]["ms"]
        line = {"metric": METRIC, "value": dv["min_sum"]["mbps"] / 1e3, "unit": UNIT, "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": dv["workload"], "l2": "flushed before every step"}, "dvbs2": dv}  # fmt: skip
    elif args.workload == "served":
        sv = measure_served(args, dist)
        line = {"metric": METRIC, "value": sv["saturation"]["gbps"], "unit": UNIT, "n_gpus": 1, "steps": 1,
                "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": sv["workload"]}, "served": sv}  # fmt: skip
    else:
        s = measure_single(args, dist, args.workload)
        line = {"metric": METRIC, "value": s["value"], "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": s["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
                "config": {"workload": s["workload"], "parallelism": f"replicas x{dist.world}"},
                "e2e": {"value": s["e2e"]["value"], "unit": UNIT, **{k: v for k, v in s["e2e"].items() if k != "value"}},
                "gpu_launches": 2 * args.steps, "roofline": s["roofline"], "demapper": s["demapper"],
                "decode": s["decode"], "parity": s["parity"]}  # fmt: skip
    if dist.rank == 0:
        if not args.no_cpu_baseline and args.workload not in ("served", "dvbs2", "mpoint", "demapper", "montecarlo"):
            sample, threads, desc = cpu_sample(args, 10.0)
            t, bits = oracle_step(sample, args.w["max_it"], threads, args.w.get("method", "maxlog"))
            line["cpu_baseline"] = {"value": bits / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                                    "sample": f"{desc}, demap + decode ({t:.1f} s)"}  # fmt: skip
        if args.workload == "mixed" and not args.no_configs and dist.world == 1:
            configs = {}
            for key, fn in (("3", lambda: measure_single(args, dist, "C")),
                            ("1", lambda: measure_single(args, dist, "A")),
                            ("2", lambda: measure_demapper(dist)),
                            ("2_mpoint", lambda: measure_mpoint(dist)),
                            ("reference_ldpc_benchmark", lambda: measure_dvbs2(dist)),
                            ("host_overhead", lambda: measure_host_overhead(dist)),
                            ("f1_montecarlo", lambda: measure_montecarlo(dist)),
                            ("5", lambda: measure_served(args, dist))):  # fmt: skip
                try:
                    configs[key] = fn()
                except Exception as exc:  # report it and keep the headline line
                    configs[key] = {"error": f"{type(exc).__name__}: {exc}"}
            line["configs"] = configs
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
