"""Several GPUs on one workload: rays and views are independent and the scene
is read-only, so each rank holds the whole scene and tree and renders its
share; rank 0 gathers the 8-bit images (and, on request, the hits) on the
host. No device collective is involved.

  * one view: contiguous bands of image rows (ho_render_tile), sizes
    differing by at most one row;
  * many views: whole views, dealt greedily by query count (largest first,
    each to the least-loaded rank), so the ranks' ray counts stay close.

The split and the gather are pure host logic (numpy + torch.distributed on
any backend); the tests run them on two gloo processes.
"""
from __future__ import annotations

import numpy as np


def row_band(height: int, world: int, rank: int) -> tuple[int, int]:
    """(first row, row count) of rank's band: contiguous, in rank order."""
    base, extra = divmod(height, world)
    y0 = rank * base + min(rank, extra)
    return y0, base + (1 if rank < extra else 0)


def view_split(queries_per_view, world: int) -> list[list[int]]:
    """Views per rank, each list in view order: largest view first to the rank
    with the fewest queries so far (ties: lowest rank, lowest view index)."""
    q = np.asarray(queries_per_view, np.int64)
    load = np.zeros(world, np.int64)
    out: list[list[int]] = [[] for _ in range(world)]
    for v in sorted(range(q.size), key=lambda i: (-int(q[i]), i)):
        r = int(np.argmin(load))
        out[r].append(v)
        load[r] += q[v]
    return [sorted(x) for x in out]


def _gather_bytes(local: np.ndarray, world: int, rank: int):
    """Rank 0 receives every rank's byte buffer (variable sizes); others get
    None. Sizes are exchanged first, buffers padded to the largest."""
    import torch
    import torch.distributed as dist

    flat = np.ascontiguousarray(local).reshape(-1).view(np.uint8)
    n = torch.tensor([flat.size], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n)
    m = max(1, int(max(int(s.item()) for s in sizes)))
    buf = torch.zeros(m, dtype=torch.uint8)
    buf[: flat.size] = torch.from_numpy(flat.copy())
    bufs = [torch.zeros(m, dtype=torch.uint8) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, bufs, dst=0)
    if rank != 0:
        return None
    return [b[: int(s.item())].numpy() for b, s in zip(bufs, sizes)]


def gather_rows(local: np.ndarray, height: int, world: int, rank: int) -> np.ndarray | None:
    """local: this rank's band, shape (n_iso, rows, W, ...). Rank 0 returns
    the whole (n_iso, height, W, ...) array, the other ranks None."""
    parts = _gather_bytes(local, world, rank)
    if rank != 0:
        return None
    n_iso, _, width = local.shape[:3]
    tail = local.shape[3:]
    out = np.zeros((n_iso, height, width) + tail, local.dtype)
    for r, raw in enumerate(parts):
        y0, rows = row_band(height, world, r)
        out[:, y0:y0 + rows] = raw.view(local.dtype).reshape((n_iso, rows, width) + tail)
    return out


def gather_views(local_parts: list[np.ndarray], assignment: list[list[int]], world: int, rank: int):
    """local_parts: this rank's per-view arrays (in its assignment order).
    Rank 0 returns all views' arrays concatenated in view order (the layout
    of a single multi-view call), the other ranks None."""
    dt = local_parts[0].dtype if local_parts else np.dtype(np.uint8)
    mine = np.concatenate([np.ascontiguousarray(p).reshape(-1).view(np.uint8) for p in local_parts]) \
        if local_parts else np.zeros(0, np.uint8)
    sizes = np.array([p.nbytes for p in local_parts], np.int64)
    parts = _gather_bytes(mine, world, rank)
    all_sizes = _gather_bytes(sizes, world, rank)
    if rank != 0:
        return None
    by_view = {}
    for r in range(world):
        raw, sz = parts[r], all_sizes[r].view(np.int64)
        off = 0
        for v, n in zip(assignment[r], sz):
            by_view[v] = raw[off:off + n]
            off += n
    return np.concatenate([by_view[v] for v in sorted(by_view)]).view(dt)
