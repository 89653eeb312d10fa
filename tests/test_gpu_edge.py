"""Edge cases of the engine through the C ABI: empty and ragged inputs, rays
that start inside the mesh or miss it, the largest isovalue count, size
limits, calls of changing sizes on one context (the per-call CUDA graph is
patched or rebuilt), and argument checks."""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
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
    Those shared-face ties are counted apart; every other ray must agree."""
    ctx, w, osc = small
    rng = np.random.default_rng(5)
    for n in (1, 31, 333, 2049):
        o = rng.uniform(-0.3, 1.3, (n, 3))
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays = np.concatenate([o, d], axis=1).astype(np.float32)
        ctx.set_mode(MODES[mode])
        h = ctx.intersect(rays, w.isovalues[0], True)
        ctx.set_mode(hr.MODE_BATCHED)
        ref, _ = osc.trace(rays, w.isovalues[0], True, precision=64)
        same = classify(h, ref)
        tie = ~same & (h["kind"] == hr.HIT_FACE) & (ref["kind"] == hr.HIT_FACE) & (np.abs(h["t"] - ref["t"]) < 2e-4)
        other = ~same & ~tie
        print(f"{mode} n={n}: shared-face ties {int(tie.sum())}, other differences {int(other.sum())}")
        assert other.sum() <= max(1, int(0.005 * n)), (n, int(other.sum()))
        m = same & (ref["kind"] > 0)
        if m.any():
            assert np.abs(h["t"][m] - ref["t"][m]).max() < 2e-4


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
