"""The benchmark's multi-rank path on the CPU (gloo, world size 2).

Rays and views are independent and the scene is read-only, so N GPUs run N
replicas: the only cross-rank steps are the barrier around the timed region,
the maximum of the ranks' times and the sum of their queries. These tests run
those helpers in two processes, and the reference arm under torchrun, where
rank 0 alone times the CPU baseline and prints the one JSON line."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist

    r, w = bench.dist_init(world)
    assert (r, w) == (rank, world)
    bench.barrier(w)
    mx = bench.max_over_ranks(1.5 + rank, w)       # per-rank time
    sm = bench.sum_over_ranks(1000 * (rank + 1), w)  # per-rank queries
    bench.barrier(w)
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"max": mx, "sum": sm}))


def test_rank_reductions_gloo(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        got = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert got == {"max": 2.5, "sum": 3000.0}  # every rank sees the job-wide figures


def test_reference_arm_two_ranks_prints_one_line():
    if not (ROOT / "oracle" / "_build" / "libhorender_oracle.so").exists():
        pytest.skip("oracle not built (oracle/Makefile)")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--gpus", "2",
           "--impl", "reference", "--workload", "prims_sheet", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
