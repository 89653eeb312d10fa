"""GPU parity against the oracle on the small curved-hex workload (hex4_p4:
4x4x4 hexes, P=4, curving 0.05h, iso 0.2), through the C ABI.

Against the FP64 oracle running the same algorithm (tests/parity.py):
  * every ray whose hit identity (kind, element, face) differs is a tie, a
    grazing ray or a ray at a decision boundary of the algorithm (classes
    counted and printed); no other difference is allowed;
  * t (the hit position along the unit ray), xi and u of the agreeing hits
    within 1e-5 of the element size / 1e-5 / 1e-5 of the oracle's hits
    polished to the exact roots of their equations;
  * padded element boxes within 1e-5 of the FP64 oracle's boxes.
"""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import parity
from conftest import classify, scene_arrays_from_ctx

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(oracle):
    ctx, w = hr.workload_context("hex4_p4")
    arrs = scene_arrays_from_ctx(ctx)
    return ctx, w, arrs, oracle.OracleScene(arrs)


def test_boxes_match_oracle(small):
    ctx, w, arrs, osc = small
    gb = ctx.boxes()
    ob = osc.boxes(64)
    assert np.abs(gb - ob).max() < 1e-5


def test_hull_contains_element(small):
    ctx, w, arrs, osc = small
    hull, faces = ctx.hull_boxes()
    boxes = ctx.boxes()
    # the padded sampled box contains the rigorous hull on this mesh
    assert (boxes[:, :3] <= hull[:, :3] + 1e-6).all() and (boxes[:, 3:] >= hull[:, 3:] - 1e-6).all()
    # the hull contains densely sampled points of each element
    rng = np.random.default_rng(0)
    xi = rng.uniform(-1, 1, (512, 3))
    for e in range(arrs.n):
        x = osc.map_point(e, xi)
        assert (x >= hull[e, :3] - 1e-6).all() and (x <= hull[e, 3:] + 1e-6).all()


@pytest.mark.parametrize("iso_on", [True, False])
def test_render_hits_match_oracle(small, oracle, iso_on):
    ctx, w, arrs, osc = small
    W = H = 128
    _, hits = ctx.render(w.camera, w.isovalues, W, H, iso_zero_disables=True, want_rgb=False, want_hits=True) \
        if iso_on else ctx.render(w.camera, [0.0], W, H, iso_zero_disables=True, want_rgb=False, want_hits=True)
    h = hits[0].reshape(-1)
    rays = oracle.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
    iso = w.isovalues[0] if iso_on else 0.0
    parity.check_against_oracle(h, rays, osc, iso, iso_on, 0.25, label=f"hex4 render iso {iso_on}",
                                product_trace=lambda r: ctx.intersect(r, iso, iso_on))


def test_plain_and_batched_modes_agree(small):
    ctx, w, arrs, osc = small
    W = H = 96
    ctx.set_mode(hr.MODE_PLAIN)
    _, hp = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    sp = ctx.stats()
    ctx.set_mode(hr.MODE_BATCHED)
    _, hb = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    same = classify(hp[0].reshape(-1), hb[0].reshape(-1))
    assert same.mean() >= 0.999
    assert sp["rays"] == W * H


@pytest.mark.parametrize("mode", ["batched", "learned"])
def test_tensor_core_and_cuda_core_rounds_agree(small, mode):
    """The tensor-core round kernel (TF32 hi/lo MMAs for the first contraction)
    and the FP32 CUDA-core kernel run the same solves; their answers differ
    only by rounding, so hit identity agrees on >= 99.9% of rays and t within
    the solvers' tolerance where it does."""
    ctx, w, arrs, osc = small
    W = H = 96
    if mode == "learned":
        ctx.train_mlp(n_samples=200_000, steps=300, batch=2048, lr=2e-3, seed=3)
        ctx.set_mode(hr.MODE_LEARNED)
    else:
        ctx.set_mode(hr.MODE_BATCHED)
    try:
        ctx.set_option(hr.OPT_TENSOR, 0)
        _, h0 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
        ctx.set_option(hr.OPT_TENSOR, 1)
        _, h1 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
        s1 = ctx.stats()
    finally:
        ctx.set_option(hr.OPT_TENSOR, 0)
        ctx.set_mode(hr.MODE_BATCHED)
    a, b = h0[0].reshape(-1), h1[0].reshape(-1)
    same = classify(a, b)
    assert same.mean() >= 0.999, f"identity agreement {same.mean():.4f}"
    m = same & (a["kind"] > 0)
    assert np.abs(a["t"][m] - b["t"][m]).max() < 2e-4
    assert s1["status"] == 0 and s1["fp64_failed_after_fallback"] == 0


def test_intersect_explicit_rays_matches_render(small):
    ctx, w, arrs, osc = small
    W = H = 64
    _, hits = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    import oracle_bind as ob

    rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
    h2 = ctx.intersect(rays, w.isovalues[0], True)
    h1 = hits[0].reshape(-1)
    same = classify(h1, h2)
    assert same.mean() > 0.999


def test_graph_rounds_and_chunks_give_the_same_hits(small):
    """The same render as a CUDA graph, as direct launches, with one round per
    launch (every further round through the completion check) and with small
    element batches: identical hits, identical work."""
    ctx, w, arrs, osc = small
    W = H = 64
    ctx.set_mode(hr.MODE_BATCHED)

    def run():
        _, h = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
        return h[0].reshape(-1).copy(), ctx.stats()

    ctx.set_option(hr.OPT_GRAPH, 0)
    h0, s0 = run()
    assert s0["graph"] == 0 and s0["rounds"] > 1 and s0["round_pairs"] <= s0["candidates"]
    ctx.set_option(hr.OPT_GRAPH, 1)
    run()
    h1, s1 = run()
    assert s1["graph"] == 1
    ctx.set_option(hr.OPT_ROUNDS, 1)
    h2, s2 = run()
    ctx.set_option(hr.OPT_ROUNDS, 16)
    ctx.set_option(hr.OPT_ROUND_CHUNK, 5)
    h3, s3 = run()
    ctx.set_option(hr.OPT_ROUND_CHUNK, 16)
    # event timing of the round kernels, inside the graph and direct
    ctx.set_option(hr.OPT_TIME_ROUNDS, 1)
    h4, s4 = run()
    assert s4["graph"] == 1 and s4["round_kernel_ns"] > 0 and s4["round_launches"] >= s4["rounds"]
    # classify, init, finish, check + fallback, and per round 6 set-up kernels + 1 round kernel
    assert s4["kernel_launches"] >= 5 + 7 * s4["round_launches"]
    ctx.set_option(hr.OPT_GRAPH, 0)
    h5, s5 = run()
    assert s5["graph"] == 0 and s5["round_kernel_ns"] > 0
    ctx.set_option(hr.OPT_GRAPH, 1)
    ctx.set_option(hr.OPT_TIME_ROUNDS, 0)
    h6, s6 = run()
    assert s6["round_kernel_ns"] == 0 and s6["round_launches"] == 0
    for h, s in ((h1, s1), (h2, s2), (h3, s3), (h4, s4), (h5, s5), (h6, s6)):
        assert np.array_equal(h["kind"], h0["kind"]) and np.array_equal(h["elem"], h0["elem"])
        assert np.array_equal(h["face"], h0["face"]) and np.array_equal(h["t"], h0["t"])
        assert (s["candidates"], s["newton_iters"], s["face_iters"]) == (
            s0["candidates"], s0["newton_iters"], s0["face_iters"])
        if s is not s2:  # one round before the tail leaves more rays to it
            assert (s["rounds"], s["round_pairs"], s["tail_rays"]) == (s0["rounds"], s0["round_pairs"], s0["tail_rays"])


@pytest.mark.parametrize("mode", ["batched", "learned"])
def test_tail_gives_the_same_hits(small, mode):
    """Rays finished by the warp-per-ray tail get the answers the rounds
    would have, with the tail after 1 or 2 rounds and without a tail
    (batched): the same hit kind, element, face and t; xi and u within 1e-5
    (the face Newton of the two kernels rounds differently in the last bits
    on a few rays). Learned: a tail
    that starts before the 4th round also takes network starts, and the
    warp-per-ray kernel restarts a missed warm sample from its converged
    neighbours where the round kernel restarts cold, so the answers agree to
    the solvers' tolerance."""
    ctx, w, arrs, osc = small
    W = H = 80
    if mode == "learned":
        ctx.train_mlp(n_samples=200_000, steps=300, batch=2048, lr=2e-3, seed=4)
        ctx.set_mode(hr.MODE_LEARNED)
    else:
        ctx.set_mode(hr.MODE_BATCHED)
    runs = []
    try:
        for tail in (0, 1, 2):
            ctx.set_option(hr.OPT_TAIL, tail)
            _, h = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
            runs.append((h[0].reshape(-1).copy(), ctx.stats()))
    finally:
        ctx.set_option(hr.OPT_TAIL, 4)
        ctx.set_mode(hr.MODE_BATCHED)
    (h0, s0), (h1, s1), (h2, s2) = runs
    assert s0["tail_rays"] == 0 and s1["tail_rays"] > 0 and s1["tail_rays"] >= s2["tail_rays"]
    for h, s in ((h1, s1), (h2, s2)):
        if mode == "batched":
            for k in ("kind", "elem", "face", "t"):
                assert np.array_equal(h[k], h0[k]), k
            assert np.abs(h["xi"] - h0["xi"]).max() < 1e-5 and np.abs(h["u"] - h0["u"]).max() < 1e-5
            assert s["candidates"] == s0["candidates"]
        else:
            same = classify(h, h0)
            assert same.mean() >= 0.999
            m = same & (h0["kind"] > 0)
            assert np.abs(h["t"][m] - h0["t"][m]).max() < 2e-4


def test_autotune_picks_a_candidate_and_keeps_results(small):
    ctx, w, arrs, osc = small
    W = H = 64
    ctx.set_mode(hr.MODE_BATCHED)
    _, h0 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    r = ctx.autotune(w.camera, w.isovalues, W, H)
    assert r["chunk"] in r["candidates"] and all(m > 0 for m in r["ms"])
    assert ctx.get_option(hr.OPT_ROUND_CHUNK) == r["chunk"]
    _, h1 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    assert np.array_equal(h0["elem"], h1["elem"]) and np.array_equal(h0["t"], h1["t"])
    ctx.set_option(hr.OPT_ROUND_CHUNK, 16)


def test_fp64_check_and_plain_fallback(small):
    """Every hit is re-evaluated in FP64; a hit that fails is traced again by
    the plain solver. With the check on, the rays that were re-traced equal
    plain mode's answers and every other ray has the unchecked answer's
    identity (or, where two hits claimed one surface point, the FP64 tie
    rule's choice), with t, xi and u polished to the exact root."""
    ctx, w, arrs, osc = small
    W = H = 96
    ctx.set_mode(hr.MODE_BATCHED)
    ctx.set_option(hr.OPT_FP64_CHECK, 0)
    _, h0 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    s0 = ctx.stats()
    ctx.set_option(hr.OPT_FP64_CHECK, 1)
    _, h1 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    s1 = ctx.stats()
    ctx.set_mode(hr.MODE_PLAIN)
    _, hp = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    ctx.set_mode(hr.MODE_BATCHED)
    h0, h1, hp = h0.reshape(-1), h1.reshape(-1), hp.reshape(-1)
    assert s0["fp64_checked"] == 0
    assert s1["fp64_checked"] == int((h0["kind"] > 0).sum())
    fb = (h1["flags"] & hr.FLAG_FALLBACK) != 0
    print("fp64: checked", s1["fp64_checked"], "failed", s1["fp64_failed"], "failed after fallback",
          s1["fp64_failed_after_fallback"])
    assert int(fb.sum()) == s1["fp64_failed"]
    assert s1["fp64_failed"] <= max(2, s1["fp64_checked"] // 100)
    # rays the FP64 tie rule weighed keep the unchecked answer unless the
    # displaced hit won; every other ray keeps it outright
    tie = (h1["flags"] & hr.FLAG_TIE) != 0
    print("fp64 tie rule: weighed", s1["fp64_ties"], "partner won", s1["fp64_ties_swapped"])
    keep = ~fb & ~tie
    for k in ("kind", "elem", "face"):
        assert np.array_equal(h1[k][fb], hp[k][fb])
        assert np.array_equal(h1[k][keep], h0[k][keep])
    swapped = ~fb & tie & ~parity.same_ids(h1, h0)
    assert int(swapped.sum()) <= s1["fp64_ties_swapped"]
    # the check polishes the hits it passes: t moves by at most the solvers'
    # tolerance, to the exact root (test_gpu_golden holds it to the judge)
    assert np.abs(h1["t"][~fb] - h0["t"][~fb]).max() < 2e-2  # the polish's step limit
    assert s1["fp64_polished"] > 0.9 * s1["fp64_checked"]
    failed_final = (h1["flags"] & hr.FLAG_FP64_FAIL) != 0
    assert int(failed_final.sum()) == s1["fp64_failed_after_fallback"]


def test_fp64_check_residuals_match_oracle(small, oracle):
    """The final check's residuals (double-single inner sums, FP64 outer sums)
    equal the FP64 oracle's x(xi) and u(xi) at the returned hits to 1e-10."""
    ctx, w, arrs, osc = small
    W = H = 64
    ctx.set_mode(hr.MODE_BATCHED)
    _, hits = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    h = hits[0].reshape(-1)
    rays = oracle.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
    res = ctx.hit_residuals(rays, h)
    hit = np.nonzero(h["kind"] > 0)[0]
    assert hit.size > 100 and (res[h["kind"] == 0] == 0).all()
    r32 = rays.astype(np.float32).astype(np.float64)
    worst_x = worst_u = 0.0
    for e in np.unique(h["elem"][hit]):
        idx = hit[h["elem"][hit] == e]
        xi = h["xi"][idx].astype(np.float64)
        x = osc.map_point(int(e), xi)
        p = r32[idx, :3] + h["t"][idx].astype(np.float64)[:, None] * r32[idx, 3:]
        rpos = np.abs(x - p).max(axis=1)
        worst_x = max(worst_x, float(np.abs(rpos - res[idx, 0]).max()))
        u = osc.eval_point(int(e), xi)[:, 9]
        worst_u = max(worst_u, float(np.abs(u - res[idx, 1]).max()))
    assert worst_x < 1e-10 and worst_u < 1e-10, (worst_x, worst_u)
    # every checked hit passes the tolerances it was checked against
    face = h["kind"][hit] == hr.HIT_FACE
    assert (res[hit[face], 0] <= 1.5e-4).all() and (res[hit[~face], 0] <= 1e-4).all()


@pytest.fixture(scope="module")
def mixed(oracle):
    """Mixed orders: 5^3 hexes with P drawn from 2..8 (modes 3..9 per element)."""
    ctx = hr.Context(0)
    ctx.generate_synthetic(5, 5, 5, 2, 8, 0.1, 32, 21)
    ctx.build_bvh()
    arrs = scene_arrays_from_ctx(ctx)
    return ctx, arrs, oracle.OracleScene(arrs)


def mixed_h(arrs):
    return 0.2  # 5 hexes per side of [0,1]^3


@pytest.mark.parametrize("tensor", [0, 1])
@pytest.mark.parametrize("iso_on", [True, False])
def test_mixed_orders_match_oracle(mixed, oracle, iso_on, tensor):
    """tensor = 1: orders 3..8 run the tensor-core round kernel, order 9 the
    CUDA-core one, in the same call."""
    ctx, arrs, osc = mixed
    assert len(set(arrs.geom_modes[:, 0].tolist())) >= 5
    cam = hr.Camera((2.5, 2.0, 1.8), (0.5, 0.5, 0.5))
    W = H = 96
    iso = 0.1 if iso_on else 0.0
    ctx.set_mode(hr.MODE_BATCHED)
    ctx.set_option(hr.OPT_TENSOR, tensor)
    try:
        _, hits = ctx.render(cam, [iso], W, H, iso_zero_disables=True, want_rgb=False, want_hits=True)
    finally:
        ctx.set_option(hr.OPT_TENSOR, 0)
    h = hits[0].reshape(-1)
    rays = oracle.camera_rays(cam.lookfrom, cam.lookat, cam.vup, cam.vfov_deg, W, H)

    def trace(r):
        ctx.set_option(hr.OPT_TENSOR, tensor)
        try:
            return ctx.intersect(r, iso, iso_on)
        finally:
            ctx.set_option(hr.OPT_TENSOR, 0)

    parity.check_against_oracle(h, rays, osc, iso, iso_on, mixed_h(arrs), product_trace=trace,
                                label=f"mixed orders, iso {iso_on}, tensor {tensor}")
    # the padded warp-per-ray engine (plain mode) gives the same answers
    ctx.set_mode(hr.MODE_PLAIN)
    _, hp = ctx.render(cam, [iso], W, H, iso_zero_disables=True, want_rgb=False, want_hits=True)
    ctx.set_mode(hr.MODE_BATCHED)
    assert classify(h, hp[0].reshape(-1)).mean() >= 0.999


@pytest.mark.parametrize("mode", [hr.MODE_BATCHED, hr.MODE_PLAIN])
def test_render_views_equals_single_views(small, mode):
    """Three views of different sizes and isovalue sets in one call equal the
    three single-camera renders (same rays, same answers)."""
    ctx, w, arrs, osc = small
    ctx.set_mode(mode)
    cams = [hr.Camera((2.5, 2.0, 1.8), (0.5, 0.5, 0.5)), hr.Camera((-1.5, 1.2, 2.2), (0.5, 0.5, 0.5), vfov_deg=45.0),
            hr.Camera((0.5, 3.0, 0.5), (0.5, 0.5, 0.5), vup=(0.0, 0.0, 1.0))]
    sizes = [(48, 32), (40, 40), (24, 56)]
    isos = [[0.2], [0.0, -0.1], [0.1, 0.2, 0.3]]
    rgb, hits, offs = ctx.render_views(cams, [s[0] for s in sizes], [s[1] for s in sizes], isos,
                                       iso_zero_disables=True, want_hits=True)
    assert offs[-1] == hits.size
    for v, (cam, (W, H), iv) in enumerate(zip(cams, sizes, isos)):
        r1, h1 = ctx.render(cam, iv, W, H, iso_zero_disables=True, want_hits=True)
        hv = hits[offs[v]:offs[v + 1]]
        assert np.array_equal(hv["elem"], h1.reshape(-1)["elem"]) and np.array_equal(hv["t"], h1.reshape(-1)["t"])
        assert np.array_equal(rgb[offs[v]:offs[v + 1]], r1.reshape(-1, 3))
    ctx.set_mode(hr.MODE_BATCHED)


def test_uneven_multiview_matches_oracle(mixed, oracle):
    """The uneven-work configuration at small scale: mixed orders, 8 seeded
    sphere views of different resolutions and 1-4 isovalues each, all in one
    call, batched and learned, against the FP64 oracle view by view: every
    identity difference classified (tests/parity.py), errors within the
    bounds."""
    ctx, arrs, osc = mixed
    cams, ws, hs, isos = hr.sphere_views(n_views=8, seed=3, shrink=16)
    ctx.train_mlp(n_samples=200_000, steps=300, batch=2048, lr=2e-3, seed=5)
    for mode in (hr.MODE_BATCHED, hr.MODE_LEARNED):
        ctx.set_mode(mode)
        _, hits, offs = ctx.render_views(cams, ws, hs, isos, want_rgb=False, want_hits=True)
        for v in range(len(cams)):
            rays = oracle.camera_rays(cams[v].lookfrom, cams[v].lookat, cams[v].vup, cams[v].vfov_deg, ws[v], hs[v])
            npix = ws[v] * hs[v]
            for k, iso in enumerate(isos[v]):
                h = hits[offs[v] + k * npix:offs[v] + (k + 1) * npix]
                # the multi-view call answers as the single-ray path on the same
                # rays (learned: a failed network start restarts from whichever
                # neighbour converged first, which the batch order decides, so
                # a ray at a decision boundary may take the other answer)
                same = classify(h, ctx.intersect(rays, iso, True))
                assert same.all() if mode == hr.MODE_BATCHED else same.mean() >= 0.999
                parity.check_against_oracle(h, rays, osc, iso, True, mixed_h(arrs),
                                            product_trace=lambda r, iso=iso: ctx.intersect(r, iso, True),
                                            label=f"multi-view mode {mode} view {v} iso {iso}")
    ctx.set_mode(hr.MODE_BATCHED)


def test_views64_scene_against_oracle(oracle):
    """The uneven-work configuration's own scene (48^3 hexes, P 2..8 per
    element) with two of its 64 sphere views at 1/8 resolution and their first
    isovalue, batched and learned: every identity difference classified and
    errors within the bounds of the FP64 judge."""
    w = hr.WORKLOADS["hex48_mixed"]
    ctx = hr.Context(0)
    try:
        ctx.generate_synthetic(**w.synth())
        ctx.build_bvh()
        ctx.train_mlp(n_samples=2_000_000, steps=600, batch=4096, lr=2e-3, seed=1)
        osc = oracle.OracleScene(scene_arrays_from_ctx(ctx))
        cams, ws, hs, isos = hr.sphere_views(n_views=64, seed=7, shrink=8)
        for mode in (hr.MODE_BATCHED, hr.MODE_LEARNED):
            ctx.set_mode(mode)
            for v in (5, 40):
                rays = oracle.camera_rays(cams[v].lookfrom, cams[v].lookat, cams[v].vup, cams[v].vfov_deg, ws[v],
                                          hs[v])
                rays = np.ascontiguousarray(rays[:: max(1, rays.shape[0] // 3000)])
                iso = isos[v][0]
                h = ctx.intersect(rays, iso, True)
                cnt = parity.check_against_oracle(h, rays, osc, iso, True, 1.0 / w.nx,
                                                  product_trace=lambda r, iso=iso: ctx.intersect(r, iso, True),
                                                  label=f"views64 scene, mode {mode}, view {v}, iso {iso}")
                assert (h["kind"] > 0).sum() > 100 and cnt["rays"] == rays.shape[0]
    finally:
        ctx.close()
