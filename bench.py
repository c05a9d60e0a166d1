"""Benchmark of the receiver back end: decoded info Gb/s at bit-identical FER.

``python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]``

Workload (the large single-code configuration): code C, a seeded 46 x 68
QC-LDPC base matrix lifted by Z = 384 (N = 26112, K = 8448), 4096 frames of
Gray 16-QAM at Eb/N0 = 1.0 dB, max-log LLRs, ``MinSum(max_iterations=50)``
with early stop.  One step = demap all 26.7 M symbols (``compute_llr``) and
decode all 4096 frames (``decode``) on the GPU.  Inputs are seeded synthetic
data (``commkit_gb300.workloads``), drawn on the host and copied to HBM.

* ``value``: decoded info bits per second over the K timed steps, inputs
  already resident in HBM (CUDA events on the launching stream, a barrier
  and a synchronize on both sides, max over ranks).
* ``e2e``: the same metric through the public API from pinned host memory:
  per step the symbols are copied host -> device, demapped, decoded, and the
  whole ``DecodeResult`` (bits, a-posteriori LLRs, valid, iterations) is
  copied back.
* ``roofline``: the decoder kernel (the dominant one), timed alone;
  algorithmic HBM bytes (LLRs in, posterior out, bits, flags) against the
  measured copy bandwidth, and in ``onchip`` its shared-memory roofline
  (8 B per edge-update: one f32 read and write of the posterior).
* ``cpu_baseline``: the CPU oracle (a C restatement of the reference's
  Numba loops, OpenMP over frames) on a bounded sample of frames.
* ``parity``: a sample of frames re-decoded by the oracle; bits, LLRs,
  iterations and syndrome flags must match bit for bit.

``--impl reference`` times the reference's CPU implementation of the path
(the oracle port: neither Numba nor CuPy is available where this runs) on
the same workload and metric, with all host threads, one bounded sample of
frames per step.  Under torchrun only rank 0 runs it.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "code C (46x68 base, Z=384, N=26112, K=8448), 4096 frames, 16-QAM max-log, Eb/N0 1.0 dB, MinSum 50 it"
FRAMES = 4096
ORDER = 16
EBN0 = 1.0
MAX_IT = 50
SEED = 1
METRIC = "decoded info Gb/s at bit-identical FER"
UNIT = "Gb/s"


def parse() -> argparse.Namespace:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--frames", type=int, default=FRAMES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0)),
                "source": "measured"}  # fmt: skip
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "fallback"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")  # fmt: skip

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)  # fmt: skip
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()
        return False

    def summary(self) -> dict:
        rows = []
        for line in (self.out or "").splitlines():
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
                "reasons": reasons, "samples": len(rows)}  # fmt: skip


def cpu_decode_sample(code_tables, batch, frames: int, threads: int):
    """The oracle's demap + decode of ``frames`` frames; returns (seconds, outputs)."""
    import oracle

    row_ptr, cols, n_var, k = code_tables
    sym = batch.symbols[:frames]
    s2 = oracle.inv_s2(batch.noise_var[0])
    t0 = time.perf_counter()
    llr = oracle.llr(sym.reshape(-1), ORDER, s2, method="maxlog", threads=threads).reshape(frames, -1)
    out = oracle.decode(llr, (row_ptr, cols, n_var), k=k, max_iterations=MAX_IT, threads=threads)
    return time.perf_counter() - t0, out


def run_reference(args) -> None:
    """The reference arm: the CPU implementation on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from commkit_gb300 import workloads as W

    oracle.build()
    threads = os.cpu_count() or 1
    spec = W.CODE_C
    checks, variables = W.lift(spec.base(), spec.z)
    m, n_var = spec.mb * spec.z, spec.nb * spec.z
    row_ptr, cols, _ = oracle.schedule(checks, variables, m, n_var)
    k = n_var - m
    # A bounded sample per step: enough frames for a few seconds on all cores.
    probe = W.coded_batch(spec, threads, ORDER, EBN0, seed=SEED)
    t, _ = cpu_decode_sample((row_ptr, cols, n_var, k), probe, threads, threads)
    per_frame = t / threads
    frames = int(max(threads, min(args.frames, threads * round(4.0 / max(per_frame * threads, 1e-3)))))
    batch = W.coded_batch(spec, frames, ORDER, EBN0, seed=SEED)
    for _ in range(args.warmup):
        cpu_decode_sample((row_ptr, cols, n_var, k), batch, frames, threads)
    times = [cpu_decode_sample((row_ptr, cols, n_var, k), batch, frames, threads)[0] for _ in range(args.steps)]
    total = sum(times)
    value = frames * k * args.steps / total / 1e9
    sample = f"{frames} of the {args.frames} frames per step (demap + decode), {threads} threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "frames_per_step": frames, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "oracle C restatement of commkit's Numba CPU loops (Numba and CuPy are not installed here)",
    }  # fmt: skip
    print(json.dumps(line), flush=True)


def main() -> None:
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist

    import commkit_gb300 as ck
    from commkit_gb300 import workloads as W

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    spec = W.CODE_C
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    const = ck.Constellation.qam(ORDER)
    method = ck.MinSum(max_iterations=MAX_IT)
    frames = args.frames
    # Each rank decodes its own frames (replicas): frames do not interact.
    batch = W.coded_batch(spec, frames, ORDER, EBN0, seed=SEED + rank)
    nv = float(batch.noise_var[0])
    sym_host = torch.from_numpy(batch.symbols).pin_memory()
    sym = sym_host.to(dev)
    plan = code._plan(local)
    ws = torch.empty(plan.workspace_size(frames), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(x):
        llr = ck.compute_llr(x, noise_var=nv, constellation=const, method="maxlog")
        return ck.decode(llr, code=code, method=method, workspace=ws)

    # ---- device-resident throughput ------------------------------------
    for _ in range(args.warmup):
        res = step(sym)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            res = step(sym)
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * frames * code.k * args.steps / (ms * 1e-3) / 1e9

    iters = res.iterations.reshape(-1).cpu().numpy()
    valid = res.valid.reshape(-1).cpu().numpy()
    bits = res.bits.reshape(frames, -1)
    fer = float(np.mean(np.any(bits.cpu().numpy() != batch.info, axis=1)))

    # ---- per-kernel times (back to back, so host work overlaps) --------
    llr_keep = ck.compute_llr(sym, noise_var=nv, constellation=const, method="maxlog")
    reps = max(3, min(args.steps, 10))
    for name in ("demap", "decode"):
        fn = (lambda: ck.compute_llr(sym, noise_var=nv, constellation=const, method="maxlog")) if name == "demap" \
            else (lambda: ck.decode(llr_keep, code=code, method=method, workspace=ws))  # fmt: skip
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if name == "demap":
            demap_ms = e0.elapsed_time(e1) / reps
        else:
            decode_ms = e0.elapsed_time(e1) / reps

    # ---- end to end through the public API, host buffers ---------------
    out_bits = torch.empty((frames, code.k), dtype=torch.int8).pin_memory()
    out_llrs = torch.empty((frames, code.n), dtype=torch.float32).pin_memory()
    out_valid = torch.empty((frames, 1), dtype=torch.bool).pin_memory()
    out_iters = torch.empty((frames, 1), dtype=torch.int32).pin_memory()

    def e2e_step():
        x = sym_host.to(dev, non_blocking=True)
        r = step(x)
        out_bits.copy_(r.bits, non_blocking=True)
        out_llrs.copy_(r.llrs, non_blocking=True)
        out_valid.copy_(r.valid, non_blocking=True)
        out_iters.copy_(r.iterations, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = world * frames * code.k * args.steps / (e2e_ms * 1e-3) / 1e9
    h2d = sym_host.numel() * 8
    d2h = out_bits.numel() + out_llrs.numel() * 4 + out_valid.numel() + out_iters.numel() * 4

    # ---- parity: a sample of frames through the oracle ------------------
    import oracle

    oracle.build()
    row_ptr, cols, _ = code._schedule
    idx = np.linspace(0, frames - 1, min(32, frames)).astype(int)
    llr_np = llr_keep.reshape(frames, -1)[torch.from_numpy(idx).to(dev)].cpu().numpy()
    s2 = oracle.inv_s2(nv)
    want_llr = oracle.llr(batch.symbols[idx].reshape(-1), ORDER, s2, method="maxlog").reshape(len(idx), -1)
    ob, op_, ov, oi = oracle.decode(want_llr, (row_ptr, cols, code.num_variables), k=code.k, max_iterations=MAX_IT)
    bit_exact = (np.array_equal(llr_np, want_llr)
                 and np.array_equal(bits.cpu().numpy()[idx], ob)
                 and np.array_equal(res.llrs.reshape(frames, -1).cpu().numpy()[idx], op_)
                 and np.array_equal(valid[idx], ov) and np.array_equal(iters[idx], oi))  # fmt: skip

    # ---- roofline of the decoder ----------------------------------------
    pk = peaks()
    E = int(code.checks.size)
    alg_bytes = frames * (4 * code.n + 4 * code.n + code.k + 5)
    achieved = alg_bytes / (decode_ms * 1e-3) / 1e9
    edge_updates = float(iters.sum()) * E
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = clk.summary().get("sm_mhz") or pk["sm_max_mhz"]
    smem_peak = sm_count * 128 * sm_mhz * 1e6 / 1e9  # GB/s at the sampled clock
    smem_achieved = 8.0 * edge_updates / (decode_ms * 1e-3) / 1e9
    demap_bytes = code.n // 4 * frames * (8 + 4 * 4)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "frames": frames, "frames_per_gpu": frames,
                   "l2": "inputs larger than L2 (214 MB symbols, 428 MB LLRs per step)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms / args.steps},
        "gpu_launches": 2 * args.steps,
        "roofline": {"kernel": "ck decoder (ldpc_decode_kernel)", "bound": "hbm", "achieved": achieved,
                     "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                     "traffic": None, "peak_source": pk["source"], "launch_ms": decode_ms,
                     "algorithmic_bytes": alg_bytes,
                     "onchip": {"bound": "smem", "achieved": smem_achieved, "peak": smem_peak, "unit": "GB/s",
                                "frac": smem_achieved / smem_peak, "edge_updates": edge_updates,
                                "edge_updates_per_s": edge_updates / (decode_ms * 1e-3)}},
        "demapper": {"launch_ms": demap_ms, "achieved_gbs": demap_bytes / (demap_ms * 1e-3) / 1e9,
                     "frac": demap_bytes / (demap_ms * 1e-3) / 1e9 / pk["hbm_gbs"]},
        "decode": {"iterations_mean": float(iters.mean()), "fer": fer, "valid": int(valid.sum())},
        "parity": {"frames_checked": int(len(idx)), "bit_exact": bool(bit_exact)},
        "clocks": clk.summary(),
    }  # fmt: skip

    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        tables = (row_ptr, cols, code.num_variables, code.k)
        t, _ = cpu_decode_sample(tables, batch, threads, threads)
        n_cpu = int(max(threads, min(frames, threads * round(10.0 / max(t, 1e-3)))))
        t, _ = cpu_decode_sample(tables, batch, n_cpu, threads)
        line["cpu_baseline"] = {"value": n_cpu * code.k / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{n_cpu} frames demap + decode ({t:.1f} s)"}  # fmt: skip
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
