"""Edge cases of the engine through the C ABI: empty and ragged inputs, rays
that start inside the mesh or miss it, the largest isovalue count, size
limits, calls of changing sizes on one context (the per-call CUDA graph is
patched or rebuilt), and argument checks."""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import parity
from conftest import classify, scene_arrays_from_ctx

pytestmark = pytest.mark.gpu

MODES = {"plain": hr.MODE_PLAIN, "batched": hr.MODE_BATCHED}


@pytest.fixture(scope="module")
def small(oracle):
    ctx, w = hr.workload_context("hex4_p4")
    arrs = scene_arrays_from_ctx(ctx)
    return ctx, w, oracle.OracleScene(arrs)


@pytest.mark.parametrize("mode", list(MODES))
def test_empty_ray_array(small, mode):
    ctx, w, osc = small
    ctx.set_mode(MODES[mode])
    h = ctx.intersect(np.zeros((0, 6), np.float32), 0.2, True)
    assert h.shape == (0,)
    ctx.set_mode(hr.MODE_BATCHED)


@pytest.mark.parametrize("mode", list(MODES))
def test_rays_from_inside_and_outside_match_oracle(small, oracle, mode):
    """Random rays with origins inside and around the mesh, in random
    directions, and ragged counts (not multiples of a warp or a block).

    A ray that starts inside the mesh meets interior faces, each shared by two
    elements: the same hit point (same kind, same t) is then reported by
    whichever element's face search accepts it first, which rounding decides
    (the FP32 and FP64 oracles themselves disagree on about 3% of such rays).
    Every difference must be such a tie or another class of tests/parity.py;
    t, xi and u of the agreeing hits within the bounds of the FP64 judge."""
    ctx, w, osc = small
    rng = np.random.default_rng(5)
    for n in (1, 31, 333, 2049):
        o = rng.uniform(-0.3, 1.3, (n, 3))
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays = np.concatenate([o, d], axis=1).astype(np.float32)
        ctx.set_mode(MODES[mode])
        h = ctx.intersect(rays, w.isovalues[0], True)

        def trace(r):
            ctx.set_mode(MODES[mode])
            return ctx.intersect(r, w.isovalues[0], True)

        parity.check_against_oracle(h, rays, osc, w.isovalues[0], True, 0.25, product_trace=trace,
                                    label=f"{mode} n={n}")
        ctx.set_mode(hr.MODE_BATCHED)


@pytest.mark.parametrize("n", [0, 1, 33, 5000])
def test_soa_rays_give_the_same_hits(small, n):
    """ho_intersect_soa (6 arrays of n floats) answers as ho_intersect on the
    same rays, bit for bit, for empty and ragged counts (all fields but the
    per-hit iteration count, which the order of a round's pairs can move)."""
    ctx, w, osc = small
    rng = np.random.default_rng(7 + n)
    o = rng.uniform(-0.5, 1.5, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-6)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    a = ctx.intersect(rays, 0.2, True)
    b = ctx.intersect_soa(np.ascontiguousarray(rays.T), 0.2, True)
    assert a.shape == b.shape == (n,)
    a["iters"] = 0
    b["iters"] = 0
    assert a.tobytes() == b.tobytes()


def test_rays_pointing_away_all_miss(small):
    ctx, w, osc = small
    n = 500
    rng = np.random.default_rng(2)
    o = rng.uniform(2.0, 3.0, (n, 3))
    d = rng.uniform(0.1, 1.0, (n, 3))  # away from the unit cube
    rays = np.concatenate([o, d], axis=1).astype(np.float32)
    h = ctx.intersect(rays, w.isovalues[0], True)
    assert (h["kind"] == hr.HIT_MISS).all() and (h["elem"] == -1).all()
    assert ctx.stats()["rays"] == n


def test_eight_isovalues_and_limits(small, oracle):
    """The largest isovalue count per call; one more, or an image beyond
    2^31 queries, is refused before any GPU work."""
    ctx, w, osc = small
    iso = np.linspace(-0.6, 0.6, 8).astype(np.float32)
    W, H = 24, 20
    _, hits = ctx.render(w.camera, iso, W, H, iso_zero_disables=False, want_rgb=False, want_hits=True)
    assert hits.shape == (8, H, W)
    rays = oracle.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
    for k in (0, 3, 7):
        ref, _ = osc.trace(rays, float(iso[k]), True, precision=64)
        assert classify(hits[k].reshape(-1), ref).mean() >= 0.99
    with pytest.raises(hr.HoError) as ei:
        ctx.render(w.camera, np.zeros(9, np.float32) + 0.1, W, H)
    assert ei.value.code == -7
    with pytest.raises(hr.HoError) as ei:
        ctx.render_device(w.camera, [0.1] * 8, 1 << 15, 1 << 14, 0, None, None)
    assert ei.value.code == -7


def test_changing_sizes_on_one_context(small):
    """Calls of different sizes and isovalue counts on one context (its
    buffers grow, its CUDA graph is patched or rebuilt) give the answers a
    fresh context gives."""
    ctx, w, osc = small
    ctx.set_mode(hr.MODE_BATCHED)
    sizes = [(16, 16, [0.2]), (64, 48, [0.2, -0.1]), (8, 8, [0.3]), (64, 48, [0.2, -0.1])]
    first = {}
    for W, H, iso in sizes:
        _, h = ctx.render(w.camera, iso, W, H, iso_zero_disables=False, want_rgb=False, want_hits=True)
        key = (W, H, tuple(iso))
        if key in first:
            assert np.array_equal(first[key]["t"], h["t"]) and np.array_equal(first[key]["elem"], h["elem"])
        first[key] = h.copy()
    fresh, _ = hr.workload_context("hex4_p4")
    with fresh:
        fresh.set_mode(hr.MODE_BATCHED)
        for W, H, iso in sizes[:3]:
            _, h = fresh.render(w.camera, iso, W, H, iso_zero_disables=False, want_rgb=False, want_hits=True)
            ref = first[(W, H, tuple(iso))]
            assert np.array_equal(ref["t"], h["t"]) and np.array_equal(ref["kind"], h["kind"])


def test_residuals_argument_checks(small):
    ctx, w, osc = small
    h = np.zeros(1, hr.HIT_DTYPE)
    h["kind"] = hr.HIT_FACE
    h["elem"] = 10_000
    with pytest.raises(hr.HoError) as ei:
        ctx.hit_residuals(np.zeros((1, 6), np.float32), h)
    assert ei.value.code == -7
    assert ctx.hit_residuals(np.zeros((0, 6), np.float32), np.zeros(0, hr.HIT_DTYPE)).shape == (0, 2)


@pytest.mark.parametrize("mode", list(MODES))
def test_zero_volume_hexes_beside_good_ones(mode):
    """Two degenerate trilinear hexahedra between the camera and the block:
    one with all 8 corners at one point, one flat (zero thickness). Their
    Jacobians are singular, so their Newton iterates turn NaN and never
    converge. The call still succeeds with device status 0, every hit has a
    finite t, no hit lies on the point-like element, and every ray that does
    not meet the degenerate elements' boxes answers as in the scene without
    them."""
    base, w = hr.workload_context("hex4_p4")
    s = base.get_scene()
    with hr.Context(0) as ctx:
        ctx.add_hexes(s["corners"], s["geom_modes"], s["geom"], s["geom_offsets"], s["field_modes"], s["field"],
                      s["field_offsets"])
        point = np.tile(np.array([1.5, 1.25, 1.15], np.float32), (8, 1))
        quad = [[1.8, 0.3, 0.3], [1.8, 0.9, 0.3], [1.8, 0.9, 0.9], [1.8, 0.3, 0.9]]
        flat = np.array(quad + quad, np.float32)  # the top face on the bottom one
        ctx.add_hexes(np.stack([point, flat]), np.zeros((2, 3), np.uint32), np.zeros(0, np.float32),
                      np.array([-1, -1]), np.zeros((2, 3), np.uint32), np.zeros(0, np.float32), np.array([-1, -1]))
        ctx.build_bvh()
        n_good = s["geom_offsets"].shape[0]
        W = H = 96
        for m in (base, ctx):
            m.set_mode(MODES[mode])
        _, h0 = base.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
        _, h1 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
        st = ctx.stats()
        assert st["status"] == 0
        h0, h1 = h0.reshape(-1), h1.reshape(-1)
        hit = h1["kind"] > 0
        assert np.isfinite(h1["t"][hit]).all()
        assert not (h1["elem"][hit] == n_good).any()
        boxes = ctx.boxes()[n_good:]
        import oracle_bind as ob

        rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
        o, d = rays[:, :3].astype(np.float64), rays[:, 3:].astype(np.float64)
        meets = np.zeros(rays.shape[0], bool)
        for b in boxes:
            with np.errstate(divide="ignore", invalid="ignore"):
                t0, t1 = (b[:3] - o) / d, (b[3:] - o) / d
            meets |= np.nanmin(np.maximum(t0, t1), 1) >= np.nanmax(np.minimum(t0, t1), 1)
        assert meets.sum() > 20  # the degenerate elements are in view
        far = ~meets
        assert np.array_equal(h1["kind"][far], h0["kind"][far]) and np.array_equal(h1["elem"][far], h0["elem"][far])
    base.close()


def test_smallest_engine_limits_give_the_same_answers(small):
    """The engine at its smallest limits: one round enqueued before each
    completion check, element batches of one pair, no tail (every ray finishes
    round by round). No queue or batch limit changes an answer."""
    ctx, w, osc = small
    ctx.set_mode(hr.MODE_BATCHED)
    W = H = 80
    _, h0 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
    saved = {o: ctx.get_option(o) for o in (hr.OPT_ROUNDS, hr.OPT_ROUND_CHUNK, hr.OPT_TAIL)}
    try:
        ctx.set_option(hr.OPT_ROUNDS, 1)
        ctx.set_option(hr.OPT_ROUND_CHUNK, 1)
        ctx.set_option(hr.OPT_TAIL, 0)
        _, h1 = ctx.render(w.camera, w.isovalues, W, H, want_rgb=False, want_hits=True)
        st = ctx.stats()
    finally:
        for o, v in saved.items():
            ctx.set_option(o, v)
    print("smallest limits:", {k: st[k] for k in ("status", "rounds", "tail_rays", "fp64_polished")})
    assert st["status"] == 0 and st["rounds"] >= 2 and st["tail_rays"] == 0
    h0, h1 = h0.reshape(-1), h1.reshape(-1)
    # the default call finishes its last rays in the warp-per-ray tail, whose
    # face Newton rounds differently in the last bits: rays at a decision
    # boundary may answer differently, every other ray identically
    import oracle_bind as ob

    rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
    c = parity.classify(h1, h0, rays, osc, w.isovalues[0],
                        product_trace=lambda r: ctx.intersect(r, w.isovalues[0], True))
    print("smallest limits vs defaults:", parity.counts(c))
    assert c["other"].size == 0 and c["differ"] <= 10
    m = parity.same_hit(h0, h1) & (h0["kind"] > 0)
    assert np.abs(h0["t"][m] - h1["t"][m]).max() <= 1e-6
