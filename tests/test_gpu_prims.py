"""Prisms, quads and curved triangles on the GPU against the oracle.

The primitive kernels are compiled without multiply-add contraction and run
the reference's FP32 steps, so on the same rays they must give the FP32
oracle's answers exactly (kind, element, t, reference coordinates); the
oracle itself is pinned bit for bit to the reference (test_prims.py). The
primitive pass follows the hexahedra's engine: with both in a scene, the
expected answer is the oracle's primitive pass started from the product's
own hexahedron hits."""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import oracle_bind as ob
import prim_scenes as ps
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MODES = {"plain": hr.MODE_PLAIN, "batched": hr.MODE_BATCHED}


def golden_arrays():
    z = np.load(GOLDEN / "prims_ref.npz")
    return ob.PrimArrays(z["kind"], z["verts"], z["geom_modes"], z["geom_offset"], z["geom"], z["field_modes"],
                         z["field_offset"], z["field"]), z


def to_oracle(h):
    out = np.zeros(h.shape[0], ob.HIT_DTYPE)
    for k in ("t", "elem", "face", "kind", "xi", "n", "u"):
        out[k] = h[k]
    out["t"][h["kind"] == hr.HIT_MISS] = 0
    return out


def compare(h, ref, label):
    """Exact agreement of kind, element, t and reference coordinates; normals
    and field values to FP32 rounding."""
    same = (h["kind"] == ref["kind"]) & (h["elem"] == ref["elem"])
    hit = ref["kind"] > 0
    same &= ~hit | (h["t"] == ref["t"].astype(np.float32))
    same &= ~hit | np.all(h["xi"] == ref["xi"].astype(np.float32), axis=1)
    bad = np.where(~same)[0]
    print(f"{label}: {h.shape[0]} rays, {int(hit.sum())} hits, {bad.size} differ")
    if bad.size:
        i = bad[0]
        print("first difference", i, h[i], ref[i])
    assert bad.size == 0
    if hit.any():
        assert np.abs(h["n"][hit] - ref["n"][hit]).max() < 1e-5
        assert np.abs(h["u"][hit] - ref["u"][hit]).max() < 1e-5


@pytest.fixture(scope="module")
def prim_scene(oracle):
    arrs, z = golden_arrays()
    ctx = hr.Context(0)
    ctx.add_prim_arrays(arrs)
    ctx.build_bvh()
    return ctx, arrs, z, oracle.OraclePrims(arrs)


CAM = hr.Camera((1.6, 1.1, 1.9), (0.5, 0.2, 0.3), vfov_deg=50.0)


def test_boxes_match_oracle(prim_scene):
    ctx, arrs, z, op = prim_scene
    assert np.array_equal(ctx.prim_boxes().astype(np.float64), op.boxes(32))
    assert np.array_equal(ctx.prim_boxes(), z["ref_boxes"])


@pytest.mark.parametrize("mode", list(MODES))
def test_primitives_only_match_oracle(prim_scene, oracle, mode):
    ctx, arrs, z, op = prim_scene
    cam_rays = oracle.camera_rays(CAM.lookfrom, CAM.lookat, CAM.vup, CAM.vfov_deg, 96, 72)
    rays = np.concatenate([cam_rays, z["rays"]])
    ctx.set_mode(MODES[mode])
    h = ctx.intersect(rays, 0.3, True)
    ctx.set_mode(hr.MODE_BATCHED)
    ref = op.trace(rays, None, 32)
    assert (ref["kind"] >= hr.HIT_PRISM).mean() > 0.3
    compare(h, ref, f"primitives only, {mode}")
    for k in (hr.HIT_PRISM, hr.HIT_QUAD, hr.HIT_TRI):
        assert (h["kind"] == k).sum() > 50, k


def test_render_and_views_shade_like_oracle(prim_scene, oracle):
    ctx, arrs, z, op = prim_scene
    W, H = 80, 60
    rgb, hits = ctx.render(CAM, [0.0], W, H, iso_zero_disables=True, want_rgb=True, want_hits=True)
    rays = oracle.camera_rays(CAM.lookfrom, CAM.lookat, CAM.vup, CAM.vfov_deg, W, H)
    ref = op.trace(rays, None, 32)
    same = (hits[0].reshape(-1)["kind"] == ref["kind"]) & (hits[0].reshape(-1)["elem"] == ref["elem"])
    print("render vs oracle, primitives:", int((~same).sum()), "of", same.size, "differ")
    assert same.mean() >= 0.995
    want = oracle.shade(rays, ref).reshape(H, W, 3)
    diff = np.abs(rgb[0].astype(int) - want.astype(int)).max(axis=2)
    assert (diff[same.reshape(H, W)] <= 1).all()
    # the same view through the multi-view call
    rgb_v, hits_v, first = ctx.render_views([CAM, CAM], [W, W], [H, H], [[0.0], [0.0]], iso_zero_disables=True,
                                            want_hits=True)
    assert np.array_equal(hits_v[:W * H]["t"], hits[0].reshape(-1)["t"])
    assert np.array_equal(hits_v[W * H:]["elem"], hits[0].reshape(-1)["elem"])


def test_hexahedra_then_primitives(oracle):
    """A hexahedral block in [0, 1]^3 beside the primitives shifted to
    x in [1.1, 2.1]: the merged answer is the oracle's primitive pass started
    from the product's hexahedron hits."""
    arrs, _ = golden_arrays()
    shifted = ps.shifted(arrs, 1.1)
    hexes, w = hr.workload_context("hex4_p4")
    both = hr.Context(0)
    h_arrays = hexes.get_scene()
    both.add_hexes(h_arrays["corners"], h_arrays["geom_modes"], h_arrays["geom"], h_arrays["geom_offsets"],
                   h_arrays["field_modes"], h_arrays["field"], h_arrays["field_offsets"])
    both.add_prim_arrays(shifted)
    both.build_bvh()
    cam = hr.Camera((1.05, 1.6, 3.2), (1.05, 0.3, 0.5), vfov_deg=55.0)
    rays = oracle.camera_rays(cam.lookfrom, cam.lookat, cam.vup, cam.vfov_deg, 120, 90)
    op = oracle.OraclePrims(shifted)
    for mode in MODES.values():
        hexes.set_mode(mode)
        both.set_mode(mode)
        hex_only = hexes.intersect(rays, w.isovalues[0], True)
        merged = both.intersect(rays, w.isovalues[0], True)
        want = op.trace(rays, to_oracle(hex_only), 32)
        assert (merged["kind"] >= hr.HIT_PRISM).mean() > 0.1
        assert ((merged["kind"] == hr.HIT_FACE) | (merged["kind"] == hr.HIT_ISO)).mean() > 0.1
        compare(merged, want, f"hexahedra + primitives, mode {mode}")


def test_path_tracing_sees_primitives(prim_scene):
    ctx, arrs, z, op = prim_scene
    img, rays = ctx.path_trace(CAM, [0.0], 64, 48, spp=2, max_depth=3, seed=3)
    img2, rays2 = ctx.path_trace(CAM, [0.0], 64, 48, spp=2, max_depth=3, seed=3)
    assert np.array_equal(img, img2) and rays == rays2
    assert rays > 64 * 48 * 2  # bounces happened
    sky = ctx.render(CAM, [0.0], 64, 48)[0][0]
    assert (np.abs(img[0].astype(int) - sky.astype(int)).sum(axis=2) > 30).mean() > 0.2


def test_vtu_wedges_and_quads_render(oracle):
    ctx = hr.Context(0)
    ctx.load_vtu(str(GOLDEN / "vtu" / "nohex.vtu"))
    ctx.build_bvh()
    g = ctx.get_prims()
    arrs = ob.PrimArrays(g["kind"], g["verts"], g["geom_modes"], g["geom_offsets"], g["geom"], g["field_modes"],
                         g["field_offsets"], g["field"])
    cam = hr.Camera((2.0, 1.5, 2.5), (0.5, 0.5, 0.5))
    rays = oracle.camera_rays(cam.lookfrom, cam.lookat, cam.vup, cam.vfov_deg, 64, 64)
    h = ctx.intersect(rays, 0.0, False)
    compare(h, oracle.OraclePrims(arrs).trace(rays, None, 32), "VTU wedges and quads")


def test_stats_after_device_call_on_caller_stream(prim_scene):
    """A primitive-only scene rendered on a caller's stream: ho_get_stats,
    read straight after the call returns, waits for that stream and reports
    the finished call (counters equal to a synchronous render's, the
    primitive pass's event time present)."""
    torch = pytest.importorskip("torch")
    ctx, arrs, z, op = prim_scene
    W, H = 320, 240
    ctx.render(CAM, [0.0], W, H, iso_zero_disables=True, want_rgb=False, want_hits=True)
    want = ctx.stats()
    rgb = torch.empty(W * H * 3, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    ctx.set_option(hr.OPT_TIME_ROUNDS, 1)
    try:
        for _ in range(3):
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                ctx.render_device(CAM, [0.0], W, H, rgb.data_ptr(), None, stream.cuda_stream)
            got = ctx.stats()
            for k in ("rays", "prim_candidates", "prim_iters", "prim_flops"):
                assert got[k] == want[k], (k, got[k], want[k])
            assert got["prim_kernel_ns"] > 0
    finally:
        ctx.set_option(hr.OPT_TIME_ROUNDS, 0)
        torch.cuda.synchronize()


def test_noalloc_path_with_primitives(prim_scene, oracle):
    torch = pytest.importorskip("torch")
    ctx, arrs, z, op = prim_scene
    rays = np.ascontiguousarray(z["rays"][:4096])
    d_rays = torch.from_numpy(rays).cuda()
    d_out = torch.zeros(rays.shape[0] * hr.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.intersect_device_noalloc(rays.shape[0], d_rays.data_ptr(), 0.0, False, d_out.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    h = d_out.cpu().numpy().view(hr.HIT_DTYPE)
    compare(h, op.trace(rays, None, 32), "no-allocation path")
