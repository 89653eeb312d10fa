"""Benchmark: Mrays/s of curved-hex ray/isosurface queries on one GB300.

Workload (default): hex64_p5 — 64^3 = 262,144 hexes of [0,1]^3, P = 5
geometry and field (6^3 modes per element), sinusoidal curving 0.12 h,
seeded 64-Gaussian field; 3840x2160 pixel-centre primary rays from a pinhole
camera at (2.5, 2.0, 1.8) looking at (0.5, 0.5, 0.5), 60 deg vertical FOV;
isovalue 0.1. One step = one render = 8,294,400 ray queries; a ray query
counts as completed whether it hits a face, the isosurface, or nothing. The
learned mode (network-predicted Newton starts + element-major batching) is
the headline; the batched mode (same kernels, cold starts) and the plain mode
(one thread per ray, the reference's per-ray structure) are timed beside it.

  value  : queries/s with the scene resident in HBM, CUDA events around the
           trace call on its own stream, L2 flushed (256 MiB write) before
           every timed step, sum over K steps.
  e2e    : the same through ho_render_tile() with a host image buffer (device
           -> host copy of the 8-bit images inside the timed region; with
           several ranks the gather on rank 0 too), host clock.
  error_vs_fp64: per mode, a seeded sample of the workload's rays that meet
           the scene box, traced by the GPU and by the FP64 oracle (TEST
           INFRASTRUCTURE, used only as the judge): identity agreement, the
           classes of the differences, and the t / xi / field errors of the
           agreeing hits against the oracle's hits polished to exact roots.
  cpu_baseline / --impl reference: the oracle's FP32 port of the reference
           algorithm (same per-candidate steps, ordered candidates), all host
           threads, on a bounded random sample of the workload's queries; the
           scene comes from the oracle's own generator, so that arm loads no
           product library.

--gpus N (under torchrun): the image's rows (or, for a multi-view workload,
whole views) are split across the ranks; every rank holds the whole scene
and tree; rank 0 gathers the images on the host. Path tracing runs one
replica per rank.

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "test-_gb300"))

METRIC = "Mrays/s (hit+iso) learned-init batched vs plain Newton, same GB300, equal error"
UNIT = "Mrays/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="hex64_p5")
    ap.add_argument("--cpu-queries", type=int, default=65536,
                    help="reference arm: CPU-port queries over its timed steps together (the GPU line's "
                         "cpu_baseline entry takes at most 16,384)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default element batch size (profiling runs: fewer launches)")
    ap.add_argument("--no-error-check", action="store_true", help="skip the error_vs_fp64 block")
    ap.add_argument("--error-rays", type=int, default=4096, help="rays of the error_vs_fp64 sample")
    ap.add_argument("--tensor", type=int, default=0, choices=[0, 1],
                    help="1: tensor-core round kernel (orders up to 8), 0: FP32 CUDA-core round kernel")
    ap.add_argument("--mode", default="all", choices=["all", "plain", "batched", "learned"],
                    help="learned: learned-init + batched (the headline); batched: the same kernels with cold "
                         "starts; plain: one thread per ray, the reference algorithm's structure")
    ap.add_argument("--train-samples", type=int, default=20_000_000,
                    help="training pairs from the plain solver (the learned configuration names 20 M)")
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--width", type=int, default=0, help="override the workload's image width (profiling)")
    ap.add_argument("--height", type=int, default=0, help="override the workload's image height (profiling)")
    return ap.parse_args()


def dist_init(n):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---- algorithmic FLOPs per counted evaluation (modes n per direction) ------
def flops_geom(n):   # x and J: 3 comps x (2n^3 + 3n^2 + 4n) FMA + basis values/derivatives (3 x 8n)
    return 2 * 3 * (2 * n**3 + 3 * n**2 + 4 * n) + 3 * 8 * n


def flops_map(n):    # x only: 3 comps x (n^3 + n^2 + n) FMA + basis values (3 x 4n)
    return 2 * 3 * (n**3 + n**2 + n) + 3 * 4 * n


def flops_field(n):  # u and grad: (2n^3 + 3n^2 + 4n) FMA + basis (3 x 8n)
    return 2 * (2 * n**3 + 3 * n**2 + 4 * n) + 3 * 8 * n


# DRAM bytes (read + write) per round-kernel launch, averaged over the 4
# launches of a step, from an ncu capture of the same workload
# (dram__bytes_read.sum + dram__bytes_write.sum over the launches of two
# learned calls; the capture commands are kept with the launch-list
# summaries). Keyed by workload, image size and mode; absent -> null.
ISECT_TRAFFIC = {
    ("hex32_p6", 1920, 1080, "learned"): (424.06e6 + 26.06e6) / 4,
    ("hex64_p5", 3840, 2160, "learned"): 1540.01e6 / 8,
}
# The same for the primitive pass (prim_trace_kernel), per launch, averaged
# over 5 launches. Nearly all of it is the
# write-back of the threads' spilled stack frames, not algorithmic traffic.
PRIM_TRAFFIC = {
    ("prims_sheet", 1920, 1080): 176.53e6 + 4569.10e6,
}


def algorithmic_flops(st, n):
    # + 3x3 inverse and update per Newton iteration (about 60 flops each)
    return (st["geom_evals"] * flops_geom(n) + st["map_evals"] * flops_map(n) + st["field_evals"] * flops_field(n)
            + (st["newton_iters"] + st["face_iters"]) * 60)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- workloads and the config both arms print --------------------------------
def hex_workload(name):
    """(scene workload, views or None, path-tracing settings or None) of a
    hexahedral workload name. Pure Python: no library is loaded."""
    import workloads as wl

    if name in wl.MULTIVIEW:
        base, kw = wl.MULTIVIEW[name]
        return wl.WORKLOADS[base], wl.sphere_views(**kw), None
    if name in wl.PATHS:
        base, kw = wl.PATHS[name]
        return wl.WORKLOADS[base], None, kw
    return wl.WORKLOADS[name], None, None


def queries_per_step(w, views):
    if views:
        cams, vw, vh, visos = views
        return int(sum(a * b * len(c) for a, b, c in zip(vw, vh, visos)))
    return w.width * w.height * len(w.isovalues)


def split_name(name, world):
    if world <= 1:
        return "1 GPU"
    import workloads as wl

    if name in wl.PATHS:
        return f"{world} GPUs: one replica of the path-traced view per rank"
    what = "whole views" if name in wl.MULTIVIEW else "image rows"
    return f"{world} GPUs: {what} split across ranks, scene and tree replicated, images gathered on rank 0"


def workload_config(name, world):
    """The workload description both arms print (identical dicts)."""
    if name in PRIMS:
        cfg = PRIMS[name]
        return {"workload": name, "scene": f"prims_sheet generator (seed {cfg['seed']}, {cfg['n_side']} per side): "
                                            "prisms on a floor of quads before a wall of triangles, half curved",
                "rays": f"{cfg['width']}x{cfg['height']} pixel-centre primary rays",
                "queries_per_step": cfg["width"] * cfg["height"],
                "l2": "GPU arm: flushed (256 MiB write) before every timed step",
                "parallelism": split_name(name, world)}
    w, views, path_kw = hex_workload(name)
    if views:
        cams, vw, vh, visos = views
        rays = (f"{len(cams)} views on a radius-2.5 sphere, resolutions {sorted(set(zip(vw, vh)))}, "
                "1-4 isovalues each")
    elif path_kw:
        rays = (f"{w.width}x{w.height}, path tracing: {path_kw['spp']} jittered path(s) per pixel per step, up to "
                f"{path_kw['max_depth']} intersections per path, Lambertian bounces")
    else:
        rays = f"{w.width}x{w.height} pixel-centre primary rays"
    return {"workload": name, "mesh": f"{w.nx}^3 = {w.nx ** 3} hexes of [0,1]^3",
            "order": w.order_max if w.order_min == w.order_max else f"P in {w.order_min}..{w.order_max}",
            "curve_amp": w.curve_amp, "gaussians": w.n_gauss, "seed": w.seed, "rays": rays,
            "isovalues": "per view" if views else w.isovalues,
            "queries_per_step": None if path_kw else queries_per_step(w, views),
            "l2": "GPU arm: flushed (256 MiB write) before every timed step",
            "parallelism": split_name(name, world)}


def scaling_of(args):
    """Rows or views of a fixed workload split over the ranks: strong; path
    tracing runs one replica per rank: weak."""
    import workloads as wl

    return "weak" if args.workload in wl.PATHS else "strong"


# ---- the CPU arm: FP32 oracle port on a bounded sample --------------------------
# the GPU line's cpu_baseline entry (at most): the reference arm's sample size,
# since a query's cost is heavy-tailed and smaller samples vary widely
CPU_BASELINE_QUERIES = 65536


def oracle_scene(w):
    """The workload's scene built by the oracle's generator (no product library)."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_bind as ob

    return ob, ob.OracleScene(ob.synth_scene(**w.synth()))


def sample_queries(ob, w, views, n, rng, box_only=False):
    """n queries drawn uniformly from the workload's queries (box_only: from
    those whose ray meets the scene box [0,1]^3 widened by 0.05): rays
    (n x 6), isovalue per query."""
    if views:
        cams, vw, vh, visos = views
        sizes = np.array([a * b * len(c) for a, b, c in zip(vw, vh, visos)], np.int64)
        first = np.concatenate([[0], np.cumsum(sizes)])
        q = np.sort(rng.choice(int(first[-1]), size=n, replace=False))
        view = np.searchsorted(first, q, side="right") - 1
        rays = np.zeros((n, 6), np.float32)
        isos = np.zeros(n, np.float32)
        for v in np.unique(view):
            m = view == v
            local = q[m] - first[v]
            npix = vw[v] * vh[v]
            c = cams[v]
            r = ob.camera_rays(c.lookfrom, c.lookat, c.vup, c.vfov_deg, vw[v], vh[v])
            rays[m] = r[local % npix]
            isos[m] = np.asarray(visos[v], np.float32)[local // npix]
        return rays, isos
    cam = w.camera
    all_rays = ob.camera_rays(cam.lookfrom, cam.lookat, cam.vup, cam.vfov_deg, w.width, w.height)
    npix = all_rays.shape[0]
    pool = np.arange(npix)
    if box_only:
        o, d = all_rays[:, :3].astype(np.float64), all_rays[:, 3:].astype(np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            t0, t1 = (-0.05 - o) / d, (1.05 - o) / d
        pool = np.where(np.maximum(t0, t1).min(1) > np.minimum(t0, t1).max(1))[0]
    n_iso = len(w.isovalues)
    q = rng.choice(pool.size * n_iso, size=n, replace=False)
    return all_rays[pool[q % pool.size]], np.asarray(w.isovalues, np.float32)[q // pool.size]


def trace_sample(osc, rays, isos, threads, precision=32):
    """Oracle trace of a query sample, grouped by isovalue (0.0 is traced as a
    real isovalue, as the GPU arm does); returns the hits in sample order."""
    out = None
    for iso in np.unique(isos):
        m = isos == iso
        h, _ = osc.trace(rays[m], float(iso), True, precision=precision, threads=threads)
        if out is None:
            out = np.zeros(rays.shape[0], h.dtype)
        out[m] = h
    return out


def cpu_sample_text(n, threads, dt, path_kw):
    what = ("primary rays of the path-traced view (the port has no bounce layer)" if path_kw
            else "queries (ray x isovalue) drawn uniformly from the workload's queries")
    return (f"{n} {what}; scene from the oracle's own generator; FP32 oracle port of the reference algorithm, "
            f"{threads} threads, {dt:.1f} s")


def cpu_baseline(name, n_queries, seed=12345):
    """The oracle's FP32 port timed on n_queries sampled queries, all host threads."""
    w, views, path_kw = hex_workload(name)
    ob, osc = oracle_scene(w)
    rng = np.random.default_rng(seed)
    threads = os.cpu_count() or 1
    warm_rays, warm_isos = sample_queries(ob, w, views, 256, rng)
    trace_sample(osc, warm_rays, warm_isos, threads)  # untimed: threads and pages warm, as the reference arm's warm-up
    rays, isos = sample_queries(ob, w, views, n_queries, rng)
    t0 = time.perf_counter()
    trace_sample(osc, rays, isos, threads)
    dt = time.perf_counter() - t0
    return {"value": n_queries / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": cpu_sample_text(n_queries, threads, dt, path_kw)}


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores (the oracle's FP32 port;
    the reference's own build needs its sources, which the GPU host does not
    have). Rank 0 alone runs; the warm-up steps trace 256 queries each, the
    timed steps --cpu-queries together. No product library is loaded."""
    if rank != 0:
        return
    per = max(256, -(-args.cpu_queries // args.steps))
    if args.workload in PRIMS:
        vals, cb = [], None
        for i in range(args.warmup + args.steps):
            cb = prims_cpu_baseline(args.workload, 256 if i < args.warmup else per, seed=i)
            if i >= args.warmup:
                vals.append(cb["value"])
        v = float(len(vals) / np.sum(1.0 / np.asarray(vals)))
    else:
        w, views, path_kw = hex_workload(args.workload)
        ob, osc = oracle_scene(w)
        rng = np.random.default_rng(12345)
        threads = os.cpu_count() or 1
        n_total, t_total = 0, 0.0
        for i in range(args.warmup + args.steps):
            n = 256 if i < args.warmup else per
            rays, isos = sample_queries(ob, w, views, n, rng)
            t0 = time.perf_counter()
            trace_sample(osc, rays, isos, threads)
            dt = time.perf_counter() - t0
            if i >= args.warmup:
                n_total += n
                t_total += dt
        v = n_total / t_total / 1e6
        cb = {"cores": threads, "kind": "port", "sample": cpu_sample_text(n_total, threads, t_total, path_kw)}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": scaling_of(args),
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": workload_config(args.workload, world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cb["cores"], "kind": cb["kind"],
                             "sample": cb["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def error_vs_fp64(ctx, hr, args, w, views, modes, codes):
    """Per solver mode, args.error_rays queries (rays that meet the scene box)
    traced by the GPU and by the FP64 oracle. Identity: agreement and the
    classes of the differences (tests/parity.py). Errors of the agreeing hits
    against the oracle's hits polished to the exact roots of their equations:
    t and the isosurface position in units of the element size h, xi, u."""
    sys.path.insert(0, str(ROOT / "tests"))
    import parity

    ob, osc = oracle_scene(w)
    rng = np.random.default_rng(2024)
    rays, isos = sample_queries(ob, w, views, args.error_rays, rng, box_only=True)
    threads = os.cpu_count() or 1
    h = 1.0 / w.nx
    o64 = trace_sample(osc, rays, isos, threads, precision=64)
    judge = np.zeros_like(o64)
    for iso in np.unique(isos):
        m = isos == iso
        judge[m] = osc.polish(rays[m], o64[m], float(iso), threads=threads)
    out = {"rays": int(rays.shape[0]), "h": h, "judge": "FP64 oracle (ordered candidates), hits polished to the exact "
           "roots of their defining equations", "modes": {}}
    for mode in modes:
        ctx.set_mode(codes[mode])
        g = np.zeros(rays.shape[0], hr.HIT_DTYPE)
        for iso in np.unique(isos):
            m = isos == iso
            g[m] = ctx.intersect(rays[m], float(iso), True)
        cls = {k: 0 for k in ("differ", "tie", "grazing", "second_root", "unstable", "other")}
        for iso in np.unique(isos):
            m = np.where(isos == iso)[0]
            c = parity.counts(parity.classify(g[m], o64[m], rays[m], osc, float(iso),
                                              product_trace=lambda r, v=float(iso): ctx.intersect(r, v, True)))
            for k in cls:
                cls[k] += c[k]
        errs = parity.errors(g, judge, rays, h)
        out["modes"][mode] = {"identity_agree": float(parity.same_ids(g, o64).mean()), "identity_classes": cls,
                              "errors": errs}
    return out


def run_gpu(args, rank, world):
    import torch

    import horender as hr
    import shard

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w, views, path_kw = hex_workload(args.workload)
    multi, path = views is not None, path_kw is not None
    if args.width and args.height:
        import dataclasses

        w = dataclasses.replace(w, width=args.width, height=args.height)
    ctx = hr.Context(local)
    ctx.generate_synthetic(**w.synth())
    ctx.build_bvh()
    ctx.set_option(hr.OPT_TENSOR, args.tensor)
    info = ctx.info()
    n_iso = len(w.isovalues)
    W, H = w.width, w.height
    # this rank's share: whole views, or a band of image rows (path tracing:
    # every rank traces the whole image, replicas)
    mine = []
    if multi:
        cams, vw, vh, visos = views
        sizes = [a * b * len(c) for a, b, c in zip(vw, vh, visos)]
        mine = shard.view_split(sizes, world)[rank]
        my_views = ([cams[i] for i in mine], [vw[i] for i in mine], [vh[i] for i in mine], [visos[i] for i in mine])
        nq = int(sum(sizes[i] for i in mine))
        y0, rows = 0, H
    else:
        y0, rows = (0, H) if path else shard.row_band(H, world, rank)
        nq = W * rows * n_iso
    rgb = torch.empty(max(nq, 1) * 3, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream

    def step():
        """One step of this rank's share; returns its ray queries."""
        if multi:
            if nq:
                ctx.render_views_device(*my_views, rgb.data_ptr(), None, sp)
        elif path:
            return ctx.path_trace_device(w.camera, w.isovalues, W, H, rgb.data_ptr(), sp, iso_zero_disables=False,
                                         **path_kw)
        elif rows:
            ctx.render_tile_device(w.camera, w.isovalues, W, H, 0, y0, W, rows, rgb.data_ptr(), None, sp,
                                   iso_zero_disables=False)
        return nq

    tuned = {}

    def timed(mode):
        ctx.set_mode(mode)
        if mode != hr.MODE_PLAIN and not args.no_autotune:  # the round kernel's element batch size
            tuned[{hr.MODE_BATCHED: "batched", hr.MODE_LEARNED: "learned"}[mode]] = ctx.autotune(
                w.camera, w.isovalues, W, H)
        # CUDA events around each round's intersection launches (event nodes of the call's graph)
        ctx.set_option(hr.OPT_TIME_ROUNDS, 0 if mode == hr.MODE_PLAIN else 1)
        keys = ("round_kernel_ns", "round_launches", "round_flops", "kernel_launches")
        per = dict.fromkeys(keys, 0)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                flush.zero_()
                step()
        torch.cuda.synchronize()
        st = ctx.stats()
        barrier(world)
        torch.cuda.synchronize()
        evs = []
        rays = 0
        with ClockSampler(local) as clk:
            with torch.cuda.stream(stream):
                for _ in range(args.steps):
                    flush.zero_()
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    rays += step()
                    b.record(stream)
                    evs.append((a, b))
                    s_step = ctx.stats()  # the call has synchronised; this reads its host copy
                    for k in keys:
                        per[k] += s_step[k]
            torch.cuda.synchronize()
        barrier(world)
        total = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / 1e3, world)
        st = dict(st, timed=per)
        return total, st, clk, rays

    train = None
    if args.mode in ("all", "learned"):
        t0 = time.perf_counter()
        losses = ctx.train_mlp(n_samples=args.train_samples, steps=args.train_steps, batch=4096, lr=2e-3, seed=1)
        torch.cuda.synchronize()
        train = {"samples": args.train_samples, "steps": args.train_steps, "batch": 4096,
                 "seconds": time.perf_counter() - t0, "loss_first": float(losses[:20].mean()),
                 "loss_last": float(losses[-50:].mean())}
    results = {}
    codes = {"plain": hr.MODE_PLAIN, "batched": hr.MODE_BATCHED, "learned": hr.MODE_LEARNED}
    if args.mode != "all":
        modes = [args.mode]
    elif multi or path:  # plain (one thread per ray, padded to the largest order) would take minutes per step here
        modes = ["batched", "learned"]
    else:
        modes = ["plain", "batched", "learned"]
    for mode in modes:
        results[mode] = timed(codes[mode])
    head = "learned" if "learned" in results else ("batched" if "batched" in results else "plain")
    total_s, st, clk, rays_timed = results[head]
    if path:
        nq = rays_timed // args.steps  # ray queries of one sample pass over all bounces
    queries = sum_over_ranks(nq * args.steps, world)
    value = queries / total_s / 1e6
    launch_s = total_s / args.steps
    plain_value = queries / results["plain"][0] / 1e6 if "plain" in results else None

    def mode_summary(m):
        if m not in results:
            return None
        t, stt, _, _ = results[m]
        return {"value": queries / t / 1e6, "ms_per_step": t / args.steps * 1e3, "newton_iters": stt["newton_iters"],
                "face_iters": stt["face_iters"], "geom_evals": stt["geom_evals"]}

    # roofline of the intersection kernel. Batched / learned: the round kernel
    # counts its own algorithmic flops (each evaluation at the element's order)
    # and CUDA events around its launches give its device time over the timed
    # steps. Plain: one launch per step, flops from the work counters at the
    # scene's largest order, over the step time.
    N = info["max_modes"]
    tm = st["timed"]
    if head != "plain" and tm["round_kernel_ns"] > 0 and tm["round_launches"] > 0:
        n_launch = tm["round_launches"]
        flops = tm["round_flops"] / n_launch
        kernel_s = tm["round_kernel_ns"] * 1e-9 / n_launch
        kernel_name = "round_kernel"
    else:
        n_launch = args.steps
        flops = algorithmic_flops(st, N)
        kernel_s = launch_s
        kernel_name = "plain_kernel"
    achieved_tflops = flops / kernel_s / 1e12

    # e2e: public API, host image buffers, D2H inside the timed region; with
    # several ranks the gather of the images on rank 0 is inside it too
    host_rgb = torch.empty(max(nq, 1) * 3, dtype=torch.uint8).pin_memory()
    e2e_rays = 0
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    ctx.set_mode(codes[head])
    for _ in range(0 if args.no_e2e else args.steps):
        if multi:
            part = host_rgb.numpy()[: nq * 3]
            if nq:
                ctx.render_views(*my_views, rgb_out=part)
            if world > 1:
                shard.gather_views([part], [[r] for r in range(world)], world, rank)
        elif path:
            img, r = ctx.path_trace(w.camera, w.isovalues, W, H, iso_zero_disables=False, **path_kw)
            host_rgb.numpy()[: img.size] = img.reshape(-1)
            e2e_rays += r
        else:
            band = host_rgb.numpy()[: nq * 3].reshape(n_iso, rows, W, 3)
            if rows:
                ctx.render_tile(w.camera, w.isovalues, W, H, 0, y0, W, rows, iso_zero_disables=False, rgb_out=band)
            if world > 1:
                shard.gather_rows(band, H, world, rank)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = None if args.no_e2e else sum_over_ranks(e2e_rays if path else nq * args.steps, world) / e2e_s / 1e6
    del host_rgb

    fp32_peak = fp32_peak_tflops(torch, dev)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True,
        "scaling": scaling_of(args), "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "impl": "gb300", "mode": {"learned": "learned-init + batched", "batched": "batched (cold-start Newton)",
                                  "plain": "plain (thread per ray, cold-start Newton)"}[head],
        "plain": mode_summary("plain"),
        "batched": mode_summary("batched"),
        "speedup_vs_plain": None if plain_value is None else value / plain_value,
        "speedup_vs_batched": (value / mode_summary("batched")["value"]) if "batched" in results and head != "batched"
        else None,
        "training": train,
        "autotune": tuned,
        "config": workload_config(args.workload, world),
        "engine": {"modes_per_dir": N, "round_kernel": ("tcgen05 TF32 hi/lo MMAs + FP32 (orders <= 8)" if args.tensor
                                                        else "FP32 CUDA cores"),
                   "rank_share": (f"views {mine}" if multi else f"rows {y0}..{y0 + rows - 1}") if world > 1 else "all"},
        "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": (achieved_tflops / fp32_peak) if fp32_peak else None,
                     "traffic": ISECT_TRAFFIC.get((w.name, W, H, head)),
                     "peak_source": "FP32 FMA loop measured in this run (peaks file has HBM and bf16 only)",
                     "kernel": kernel_name, "flops_per_launch": flops, "launches": n_launch,
                     "ms_per_launch": kernel_s * 1e3,
                     "share_of_step": kernel_s * n_launch / total_s},
        "e2e": None if e2e is None else {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 44 + 4 * n_iso,
                                         "d2h_bytes_per_step": (W * H * n_iso if path else nq) * 3},
        "gpu_launches": tm["kernel_launches"],
        "clocks": clk.summary(),
        "work": st,
        "scene": info,
    }
    if rank == 0 and world == 1 and not args.no_error_check and not path:
        line["error_vs_fp64"] = error_vs_fp64(ctx, hr, args, w, views, [m for m in ("plain", "batched", "learned")
                                                                         if m in results], codes)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, min(CPU_BASELINE_QUERIES, args.cpu_queries))
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


# ---- prisms, quads and curved triangles --------------------------------------
# One scene of the three non-hexahedral primitive kinds (tents on a floor of
# quads before a wall of triangles, half of them curved), rendered primary
# rays only: every query goes through the primitive pass (the scene has no
# hexahedra). Seeded, generated on the host (prim_synth).
PRIMS = {"prims_sheet": dict(seed=11, n_side=64, width=1920, height=1080,
                             camera=((1.6, 1.1, 1.9), (0.5, 0.2, 0.3), 50.0))}


def prims_scene(name):
    import prim_synth

    cfg = PRIMS[name]
    return prim_synth.mixed_scene(seed=cfg["seed"], n_side=cfg["n_side"]), cfg


def prims_cpu_baseline(name, n_queries, seed=0):
    """The FP32 oracle's primitive pass on n_queries rays drawn from the
    workload's image, all host threads."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_bind as ob

    ps, cfg = prims_scene(name)
    arrs = ob.PrimArrays(ps.kind, ps.verts, ps.geom_modes, ps.geom_offset, ps.geom, ps.field_modes, ps.field_offset,
                         ps.field)
    op = ob.OraclePrims(arrs)
    frm, at, fov = cfg["camera"]
    rays = ob.camera_rays(frm, at, (0, 1, 0), fov, cfg["width"], cfg["height"])
    rng = np.random.default_rng(seed)
    threads = os.cpu_count() or 1
    idx = rng.choice(rays.shape[0], n_queries, replace=False)
    t0 = time.perf_counter()
    op.trace(rays[idx], None, 32, threads)
    dt = time.perf_counter() - t0
    return {"value": n_queries / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n_queries} primary rays drawn uniformly from the {cfg['width']}x{cfg['height']} image, "
                      f"FP32 oracle port of the reference's primitive routines, {threads} threads, {dt:.1f} s"}


def run_prims(args, rank, world):
    import torch

    import horender as hr

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import shard

    ps, cfg = prims_scene(args.workload)
    W, H = (args.width, args.height) if args.width and args.height else (cfg["width"], cfg["height"])
    y0, rows = shard.row_band(H, world, rank)
    frm, at, fov = cfg["camera"]
    cam = hr.Camera(frm, at, vfov_deg=fov)
    ctx = hr.Context(local)
    ctx.add_prim_arrays(ps)
    ctx.build_bvh()
    ctx.set_option(hr.OPT_TIME_ROUNDS, 1)
    info = ctx.info()
    nq = W * rows
    rgb = torch.empty(max(nq, 1) * 3, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    keys = ("prim_kernel_ns", "prim_flops", "prim_candidates", "prim_iters", "kernel_launches")
    per = dict.fromkeys(keys, 0)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            if rows:
                ctx.render_tile_device(cam, [0.0], W, H, 0, y0, W, rows, rgb.data_ptr(), None, sp)
    torch.cuda.synchronize()
    barrier(world)
    evs = []
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for _ in range(args.steps):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                if rows:
                    ctx.render_tile_device(cam, [0.0], W, H, 0, y0, W, rows, rgb.data_ptr(), None, sp)
                b.record(stream)
                evs.append((a, b))
                s_step = ctx.stats()
                for k in keys:
                    per[k] += s_step[k]
        torch.cuda.synchronize()
    barrier(world)
    total_s = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / 1e3, world)
    queries = sum_over_ranks(nq * args.steps, world)
    value = queries / total_s / 1e6
    kernel_s = per["prim_kernel_ns"] * 1e-9 / args.steps
    flops = per["prim_flops"] / args.steps
    achieved = flops / kernel_s / 1e12
    # e2e: public API, host image buffer, D2H inside the timed region
    host_rgb = torch.empty((1, rows, W, 3), dtype=torch.uint8).pin_memory()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(0 if args.no_e2e else args.steps):
        if rows:
            ctx.render_tile(cam, [0.0], W, H, 0, y0, W, rows, rgb_out=host_rgb.numpy())
        if world > 1:
            shard.gather_rows(host_rgb.numpy(), H, world, rank)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = None if args.no_e2e else queries / e2e_s / 1e6
    fp32_peak = fp32_peak_tflops(torch, dev)
    st = ctx.stats()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True,
        "scaling": scaling_of(args), "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "impl": "gb300", "mode": "primitive pass (prisms, quads, curved triangles; thread per query)",
        "config": workload_config(args.workload, world),
        "engine": {"primitives": {"prisms": info["n_prisms"], "quads": info["n_quads"], "triangles": info["n_tris"]},
                   "curved": int((ps.geom_offset >= 0).sum()),
                   "rank_share": f"rows {y0}..{y0 + rows - 1}" if world > 1 else "all"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": (achieved / fp32_peak) if fp32_peak else None,
                     "traffic": PRIM_TRAFFIC.get((args.workload, W, H)),
                     "peak_source": "FP32 FMA loop measured in this run (peaks file has HBM and bf16 only)",
                     "kernel": "prim_trace_kernel", "flops_per_launch": flops, "launches": args.steps,
                     "ms_per_launch": kernel_s * 1e3, "share_of_step": kernel_s * args.steps / total_s},
        "e2e": None if e2e is None else {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 44 + 4,
                                         "d2h_bytes_per_step": nq * 3},
        "gpu_launches": per["kernel_launches"],
        "clocks": clk.summary(),
        "work": {"candidates_per_query": per["prim_candidates"] / queries,
                 "iterations_per_query": per["prim_iters"] / queries, "last_call": st},
        "scene": info,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = prims_cpu_baseline(args.workload, min(CPU_BASELINE_QUERIES, args.cpu_queries))
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def fp32_peak_tflops(torch, dev):
    """Measured FP32 FMA rate of this GPU in TFLOP/s (ho_measure_fp32_peak)."""
    import horender as hr

    return hr.fp32_fma_peak_tflops(dev.index or 0)


def main():
    args = parse()
    rank, world = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload in PRIMS:
        run_prims(args, rank, world)
    else:
        run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
