"""Benchmark of the receiver back end: decoded info Gb/s at bit-identical FER.

``python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]``

Default workload (the large single-code configuration): code C, a seeded 46 x 68
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

# The measured configurations: code, frames, constellation, demapper method,
# Eb/N0 and MinSum iterations.  "C" (the large single-code batch) is the
# default; "A" is the plain CPU-runnable configuration.
WORKLOADS = {
    "C": dict(code="C", frames=4096, order=16, method="maxlog", ebn0=1.0, max_it=50,
              desc="code C (46x68 base, Z=384, N=26112, K=8448), 4096 frames, 16-QAM max-log, "
                   "Eb/N0 1.0 dB, MinSum 50 it"),
    "A": dict(code="A", frames=1024, order=4, method="exact", ebn0=2.5, max_it=20,
              desc="code A (12x24 base, Z=54, N=1296, K=648), 1024 frames, QPSK exact LLRs, "
                   "Eb/N0 2.5 dB, MinSum 20 it"),
    "mixed": dict(code="mixed", frames=8192, max_it=50,
                  desc="mixed batch of 8192 frames: codes A/B/C 60/30/10 (QPSK, 16-QAM, 16-QAM, "
                       "max-log), per-frame Eb/N0 within +-1 dB of each code's waterfall, MinSum 50 it"),
}  # fmt: skip
SEED = 1
METRIC = "decoded info Gb/s at bit-identical FER"
UNIT = "Gb/s"


def parse() -> argparse.Namespace:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="C")
    ap.add_argument("--frames", type=int, default=0, help="override the workload's frame count")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.w = WORKLOADS[args.workload]
    if args.frames <= 0:
        args.frames = args.w["frames"]
    return args


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


def cpu_decode_sample(w, code_tables, batch, frames: int, threads: int):
    """The oracle's demap + decode of ``frames`` frames; returns (seconds, outputs)."""
    import oracle

    row_ptr, cols, n_var, k = code_tables
    sym = batch.symbols[:frames]
    s2 = oracle.inv_s2(batch.noise_var[0])
    t0 = time.perf_counter()
    llr = oracle.llr(sym.reshape(-1), w["order"], s2, method=w["method"], threads=threads).reshape(frames, -1)
    out = oracle.decode(llr, (row_ptr, cols, n_var), k=k, max_iterations=w["max_it"], threads=threads)
    return time.perf_counter() - t0, out


def run_reference(args) -> None:
    """The reference arm: the CPU implementation on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from commkit_gb300 import workloads as W

    oracle.build()
    w = args.w
    threads = os.cpu_count() or 1
    spec = W.CODES[w["code"]]
    checks, variables = W.lift(spec.base(), spec.z)
    m, n_var = spec.mb * spec.z, spec.nb * spec.z
    row_ptr, cols, _ = oracle.schedule(checks, variables, m, n_var)
    k = n_var - m
    tables = (row_ptr, cols, n_var, k)
    # A bounded sample per step: enough frames for a few seconds on all cores.
    probe = W.coded_batch(spec, threads, w["order"], w["ebn0"], seed=SEED)
    t, _ = cpu_decode_sample(w, tables, probe, threads, threads)
    frames = int(max(threads, min(args.frames, threads * round(4.0 / max(t, 1e-3)))))
    batch = W.coded_batch(spec, frames, w["order"], w["ebn0"], seed=SEED)
    for _ in range(args.warmup):
        cpu_decode_sample(w, tables, batch, frames, threads)
    times = [cpu_decode_sample(w, tables, batch, frames, threads)[0] for _ in range(args.steps)]
    total = sum(times)
    value = frames * k * args.steps / total / 1e9
    sample = f"{frames} of the {args.frames} frames per step (demap + decode), {threads} threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "frames_per_step": frames, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "oracle C restatement of commkit's Numba CPU loops (Numba and CuPy are not installed here)",
    }  # fmt: skip
    print(json.dumps(line), flush=True)


def run_mixed(args) -> None:
    """Config 4: one mixed batch of codes A/B/C.  The batched form (demap +
    one mixed-code persistent launch, captured in a CUDA graph) against the
    plain form (the public API, one demap and one decode call per code) on
    the same frames."""
    import torch

    import commkit_gb300 as ck
    import oracle
    from commkit_gb300 import workloads as W
    from commkit_gb300.pipeline import CodeSlot, MixedReceiver

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    w = args.w
    work = W.mixed_workload(total=args.frames)
    method = ck.MinSum(max_iterations=w["max_it"])
    names = list(work)
    codes = {n: ck.LDPCCode.quasi_cyclic(W.CODES[n].base(), lifting=W.CODES[n].z) for n in names}
    consts = {n: ck.Constellation.qam(W.MIXED_ORDERS[n]) for n in names}
    slots = [CodeSlot(codes[n], consts[n], work[n].symbols.shape[0], method) for n in names]
    rx = MixedReceiver(slots, dev)
    sym_host = [torch.from_numpy(work[n].symbols).pin_memory() for n in names]
    nv = [work[n].noise_var for n in names]
    rx.load(sym_host, nv)
    rx.capture()
    info_bits = sum(int(work[n].symbols.shape[0]) * codes[n].k for n in names)

    def timed(fn, steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    for _ in range(args.warmup):
        rx.run()
    with Clocks(0) as clk:
        ms = timed(rx.run, args.steps)
    value = info_bits * args.steps / (ms * 1e-3) / 1e9
    res = rx.results()

    # Plain form: public API calls, one homogeneous batch per code.
    sym_dev = [s.to(dev) for s in sym_host]

    def plain_step():
        out = []
        for i, n in enumerate(names):
            llr = ck.compute_llr_frames(sym_dev[i], noise_var=nv[i], constellation=consts[n])
            out.append(ck.decode(llr, code=codes[n], method=method))
        return out

    for _ in range(args.warmup):
        plain = plain_step()
    plain_ms = timed(plain_step, args.steps)
    plain = plain_step()
    plain_value = info_bits * args.steps / (plain_ms * 1e-3) / 1e9
    same = all(np.array_equal(r.llrs.cpu().numpy(), p_.llrs.cpu().numpy().reshape(r.llrs.shape))
               and np.array_equal(r.bits.cpu().numpy(), p_.bits.cpu().numpy().reshape(r.bits.shape))
               and np.array_equal(r.iterations.cpu().numpy(), p_.iterations.cpu().numpy().reshape(-1))
               for r, p_ in zip(res, plain, strict=True))  # fmt: skip

    # Decoder alone: the mixed launch (captured step minus the demaps).
    e_llrs = [rx.llr[i] for i in range(len(names))]

    def dec_only():
        ck.decode_mixed([(e_llrs[i], codes[n], method) for i, n in enumerate(names)],
                        workspace=rx.workspace, outputs=rx.outputs)  # fmt: skip

    dec_ms = timed(dec_only, max(3, args.steps)) / max(3, args.steps)

    # e2e: pinned host symbols in, every result out.
    outs = [(torch.empty_like(o[0], device="cpu").pin_memory(), torch.empty_like(o[1], device="cpu").pin_memory(),
             torch.empty_like(o[2], device="cpu").pin_memory(), torch.empty_like(o[3], device="cpu").pin_memory())
            for o in rx.outputs]  # fmt: skip

    def e2e_step():
        for i in range(len(names)):
            rx.sym[i].copy_(sym_host[i], non_blocking=True)
        rx.run()
        for o_host, o_dev in zip(outs, rx.outputs, strict=True):
            for a, b in zip(o_host, o_dev, strict=True):
                a.copy_(b, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_ms = timed(e2e_step, args.steps)
    e2e_value = info_bits * args.steps / (e2e_ms * 1e-3) / 1e9
    h2d = sum(s.numel() * 8 for s in sym_host)
    d2h = sum(sum(t.numel() * t.element_size() for t in o) for o in outs)

    # Parity: 16 frames per code through the oracle (LLRs and decode).
    parity_ok = True
    fer, iters_all = {}, []
    oracle.build()
    for i, n in enumerate(names):
        F = work[n].symbols.shape[0]
        idx = np.linspace(0, F - 1, min(16, F)).astype(int)
        want = np.stack([oracle.llr(work[n].symbols[f], W.MIXED_ORDERS[n], oracle.inv_s2(work[n].noise_var[f])).reshape(-1)
                         for f in idx])  # fmt: skip
        got = rx.llr[i].cpu().numpy()[idx]
        row, col, _ = codes[n]._schedule
        ob, opost, ov, oi = oracle.decode(want, (row, col, codes[n].num_variables), k=codes[n].k,
                                          max_iterations=w["max_it"])  # fmt: skip
        r = res[i]
        parity_ok &= (np.array_equal(got, want) and np.array_equal(r.bits.cpu().numpy()[idx], ob)
                      and np.array_equal(r.llrs.cpu().numpy()[idx], opost)
                      and np.array_equal(r.iterations.cpu().numpy()[idx], oi)
                      and np.array_equal(r.valid.cpu().numpy()[idx], ov))  # fmt: skip
        it = r.iterations.cpu().numpy()
        iters_all.append((it, codes[n].checks.size))
        fer[n] = float(np.mean(np.any(r.bits.cpu().numpy() != work[n].info, axis=1)))

    pk = peaks()
    edge_updates = float(sum(it.sum() * E for it, E in iters_all))
    alg_bytes = sum(int(work[n].symbols.shape[0]) * (8 * codes[n].n + codes[n].k + 5) for n in names)
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = clk.summary().get("sm_mhz") or pk["sm_max_mhz"]
    smem_peak = sm_count * 128 * sm_mhz * 1e6 / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "frames": {n: int(work[n].symbols.shape[0]) for n in names},
                   "form": "batched: demap + one mixed-code persistent launch per step, CUDA-graph replay",
                   "l2": "inputs larger than L2"},
        "plain": {"value": plain_value, "ms_per_step": plain_ms / args.steps,
                  "form": "public API: compute_llr_frames + decode per code", "bit_identical_to_batched": bool(same)},
        "batched_over_plain": value / plain_value,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms / args.steps},
        "gpu_launches": (len(names) + 1) * args.steps,
        "roofline": {"kernel": "ck mixed decoder (ldpc_mixed_kernel)", "bound": "hbm",
                     "achieved": alg_bytes / (dec_ms * 1e-3) / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": alg_bytes / (dec_ms * 1e-3) / 1e9 / pk["hbm_gbs"], "traffic": None,
                     "peak_source": pk["source"], "launch_ms": dec_ms,
                     "onchip": {"bound": "smem", "achieved": 8 * edge_updates / (dec_ms * 1e-3) / 1e9,
                                "peak": smem_peak, "unit": "GB/s",
                                "frac": 8 * edge_updates / (dec_ms * 1e-3) / 1e9 / smem_peak,
                                "edge_updates_per_s": edge_updates / (dec_ms * 1e-3)}},
        "decode": {"fer": fer, "iterations": {n: [int(it.min()), float(it.mean()), int(it.max())]
                                             for n, (it, _) in zip(names, iters_all, strict=True)}},
        "parity": {"frames_checked": 16 * len(names), "bit_exact": bool(parity_ok)},
        "clocks": clk.summary(),
    }  # fmt: skip
    print(json.dumps(line), flush=True)


def main() -> None:
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "mixed":
        run_mixed(args)
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

    w = args.w
    spec = W.CODES[w["code"]]
    code = ck.LDPCCode.quasi_cyclic(spec.base(), lifting=spec.z)
    const = ck.Constellation.qam(w["order"])
    method = ck.MinSum(max_iterations=w["max_it"])
    demap = w["method"]
    frames = args.frames
    # Each rank decodes its own frames (replicas): frames do not interact.
    batch = W.coded_batch(spec, frames, w["order"], w["ebn0"], seed=SEED + rank)
    nv = float(batch.noise_var[0])
    sym_host = torch.from_numpy(batch.symbols).pin_memory()
    sym = sym_host.to(dev)
    plan = code._plan(local)
    ws = torch.empty(plan.workspace_size(frames), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(x):
        llr = ck.compute_llr(x, noise_var=nv, constellation=const, method=demap)
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
    llr_keep = ck.compute_llr(sym, noise_var=nv, constellation=const, method=demap)
    reps = max(3, min(args.steps, 10))
    for name in ("demap", "decode"):
        fn = (lambda: ck.compute_llr(sym, noise_var=nv, constellation=const, method=demap)) if name == "demap" \
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
    want_llr = oracle.llr(batch.symbols[idx].reshape(-1), w["order"], s2, method=demap).reshape(len(idx), -1)
    # max-log LLRs are bit-exact; exact ones agree within rtol 1e-5 / atol 1e-6.  The
    # decoder is then checked bit for bit on the GPU's own LLRs.
    llr_ok = (np.array_equal(llr_np, want_llr) if demap == "maxlog"
              else np.allclose(llr_np, want_llr, rtol=1e-5, atol=1e-6))  # fmt: skip
    ob, op_, ov, oi = oracle.decode(llr_np, (row_ptr, cols, code.num_variables), k=code.k,
                                    max_iterations=w["max_it"])  # fmt: skip
    bit_exact = (llr_ok
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
    ksym = const.bits_per_symbol
    demap_bytes = code.n // ksym * frames * (8 + 4 * ksym)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": w["desc"], "frames": frames, "frames_per_gpu": frames,
                   "l2": f"inputs {'larger' if sym_host.numel() * 8 > 129e6 else 'smaller'} than L2 "
                         f"({sym_host.numel() * 8 / 1e6:.0f} MB symbols, {frames * code.n * 4 / 1e6:.0f} MB LLRs per step)",
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
        t, _ = cpu_decode_sample(w, tables, batch, threads, threads)
        n_cpu = int(max(threads, min(frames, threads * round(10.0 / max(t, 1e-3)))))
        t, _ = cpu_decode_sample(w, tables, batch, n_cpu, threads)
        line["cpu_baseline"] = {"value": n_cpu * code.k / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{n_cpu} frames demap + decode ({t:.1f} s)"}  # fmt: skip
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
