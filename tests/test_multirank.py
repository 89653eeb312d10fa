"""The multi-rank path on the CPU (gloo, world size 2).

Rays and views are independent and the scene is read-only, so N GPUs split
one workload: contiguous bands of image rows of a single view, or whole views
of a multi-view call (test-_gb300/shard.py), every rank holding the whole
scene and tree; rank 0 gathers the images and hits on the host. The
benchmark's other cross-rank steps are the barrier around the timed region,
the maximum of the ranks' times and the sum of their queries. These tests run
the split and gather in two processes with the CPU oracle tracing each rank's
share (the gathered images and hits must equal one rank's, bit for bit), the
reductions, and the reference arm under torchrun, where rank 0 alone times
the CPU baseline and prints the one JSON line."""
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


def _oracle_scene():
    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT / "test-_gb300"))
    import oracle_bind as ob
    import workloads as wl

    w = wl.WORKLOADS["hex4_p4"]
    return ob, w, ob.OracleScene(ob.synth_scene(**w.synth()))


def _trace_rows(ob, osc, w, W, H, y0, rows):
    rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
    rays = rays.reshape(H, W, 6)[y0:y0 + rows].reshape(-1, 6)
    hits, _ = osc.trace(rays, w.isovalues[0], True, precision=32, threads=1)
    rgb = ob.shade(rays, hits)
    return rgb.reshape(1, rows, W, 3), hits.reshape(1, rows, W)


VIEWS = [((2.5, 2.0, 1.8), 21, 13), ((-1.5, 0.4, 2.2), 9, 30), ((0.4, 0.6, 3.0), 16, 16), ((2.2, -1.0, -0.8), 7, 5),
         ((-1.0, -1.5, 1.0), 25, 8)]


def _trace_view(ob, osc, w, v):
    frm, W, H = VIEWS[v]
    rays = ob.camera_rays(frm, (0.5, 0.5, 0.5), (0, 1, 0), 50.0, W, H)
    hits, _ = osc.trace(rays, w.isovalues[0], True, precision=32, threads=1)
    return ob.shade(rays, hits), hits


def _shard_main(rank, world, port, out_dir, W, H):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import torch.distributed as dist

    import bench
    import shard

    bench.dist_init(world)
    ob, w, osc = _oracle_scene()
    y0, rows = shard.row_band(H, world, rank)
    rgb, hits = _trace_rows(ob, osc, w, W, H, y0, rows)
    full_rgb = shard.gather_rows(rgb, H, world, rank)
    full_hits = shard.gather_rows(hits, H, world, rank)
    sizes = [VIEWS[v][1] * VIEWS[v][2] for v in range(len(VIEWS))]
    assign = shard.view_split(sizes, world)
    mine = [_trace_view(ob, osc, w, v) for v in assign[rank]]
    views_rgb = shard.gather_views([m[0] for m in mine], assign, world, rank)
    views_hits = shard.gather_views([m[1] for m in mine], assign, world, rank)
    dist.destroy_process_group()
    if rank == 0:
        np.savez(Path(out_dir, "gathered.npz"), rgb=full_rgb, hits=full_hits, views_rgb=views_rgb,
                 views_hits=views_hits)


def test_row_bands_and_views():
    sys.path.insert(0, str(ROOT / "test-_gb300"))
    import shard

    for H in (1, 2, 7, 37, 2160):
        for world in (1, 2, 3, 8):
            bands = [shard.row_band(H, world, r) for r in range(world)]
            assert sum(b[1] for b in bands) == H
            assert all(bands[r][0] + bands[r][1] == (bands[r + 1][0] if r + 1 < world else H) for r in range(world))
            assert max(b[1] for b in bands) - min(b[1] for b in bands) <= 1
    sizes = [5, 100, 7, 64, 64, 1, 30]
    for world in (1, 2, 3, 8):
        a = shard.view_split(sizes, world)
        assert sorted(v for part in a for v in part) == list(range(len(sizes)))
        assert all(part == sorted(part) for part in a)
    load = [sum(sizes[v] for v in part) for part in shard.view_split(sizes, 2)]
    assert max(load) - min(load) <= max(sizes)
    assert shard.view_split(sizes, 2) == shard.view_split(sizes, 2) == [[0, 1, 5, 6], [2, 3, 4]]


def test_split_and_gather_equal_one_rank_gloo(tmp_path):
    """Two gloo ranks trace their row bands (and their views) with the CPU
    oracle; rank 0's gathered images and hits equal one process's, bit for
    bit."""
    import numpy as np

    mp = pytest.importorskip("torch.multiprocessing")
    if not (ROOT / "oracle" / "_build" / "libhorender_oracle.so").exists():
        pytest.skip("oracle not built (oracle/Makefile)")
    W, H = 40, 31  # odd row count: the bands differ by one row
    port = free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_shard_main, args=(r, 2, port, str(tmp_path), W, H)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    got = np.load(tmp_path / "gathered.npz")
    ob, w, osc = _oracle_scene()
    rgb, hits = _trace_rows(ob, osc, w, W, H, 0, H)
    assert np.array_equal(got["rgb"], rgb)
    assert got["hits"].tobytes() == hits.tobytes()
    assert (hits["kind"] > 0).sum() > 100
    one = [_trace_view(ob, osc, w, v) for v in range(len(VIEWS))]
    assert np.array_equal(got["views_rgb"].reshape(-1, 3), np.concatenate([o[0] for o in one]))
    assert got["views_hits"].tobytes() == np.concatenate([o[1] for o in one]).tobytes()


def test_reference_arm_two_ranks_prints_one_line():
    if not (ROOT / "oracle" / "_build" / "libhorender_oracle.so").exists():
        pytest.skip("oracle not built (oracle/Makefile)")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--gpus", "2",
           "--impl", "reference", "--workload", "prims_sheet", "--steps", "1", "--warmup", "0",
           "--cpu-queries", "512"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
