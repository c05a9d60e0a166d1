"""bench.py's multi-rank path on CPU: two gloo ranks, as torchrun starts them.

The path shards by frames: each rank decodes its own frames (the
workload's seed includes the rank), with no exchange but the timings.  The
whole-job rate is the ranks' units over the slowest rank's time, and the
reference arm runs on rank 0 only."""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))  # fmt: skip
    sys.path.insert(0, str(REPO))
    import bench
    from commkit_gb300 import workloads as W

    dist = bench.Dist(backend="gloo")
    dist.barrier()
    slowest = dist.max(1.0 + rank)  # this rank's "ms"
    work = W.mixed_workload(total=40, seed=11 + rank)
    frames = {n: int(b.symbols.shape[0]) for n, b in work.items()}
    first = {n: b.symbols[0, :4].tolist() for n, b in work.items()}
    rate = dist.rate(1000.0, slowest)
    dist.barrier()
    dist.close()
    Path(out).write_text(json.dumps({"slowest": slowest, "frames": frames, "rate": rate,
                                     "first": {n: [[z.real, z.imag] for z in v] for n, v in first.items()}}))


def test_two_gloo_ranks(tmp_path):
    import multiprocessing as mp

    port = _free_port()
    ctx = mp.get_context("spawn")
    outs = [str(tmp_path / f"rank{r}.json") for r in range(2)]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, outs[r])) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = [json.loads(Path(o).read_text()) for o in outs]
    # max over ranks, seen by both
    assert res[0]["slowest"] == res[1]["slowest"] == 2.0
    # the same units per rank (frames per code), different frames
    assert res[0]["frames"] == res[1]["frames"]
    assert any(not np.allclose(res[0]["first"][n], res[1]["first"][n]) for n in res[0]["first"])
    # whole job: 2 ranks x 1000 units in 2 ms
    assert res[0]["rate"] == pytest.approx(2 * 1000 / 2e-3)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], cwd=REPO, env=env, capture_output=True, text=True, timeout=300)  # fmt: skip
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
