"""A scene loaded from a VTU file, rendered on the GPU against the oracle: a
generated 12x10x8 grid of jittered trilinear hexahedra (no field, so rays find
element faces only), in the plain and batched solvers, through
ho_intersect and ho_render."""
from __future__ import annotations

import sys

import numpy as np
import pytest

import horender as hr
import parity
from conftest import GOLDEN, classify, scene_arrays_from_ctx

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vtu_scene(tmp_path_factory, oracle):
    sys.path.insert(0, str(GOLDEN))
    import make_vtu as mv

    rng = np.random.default_rng(3)
    p = mv.grid_points(12, 10, 8, rng, jitter=0.25)
    hexes = mv.grid_hexes(12, 10, 8)
    conn, off = mv.flat(hexes)
    path = tmp_path_factory.mktemp("vtu") / "grid.vtu"
    path.write_text(mv.vtu(mv.fmt_points(p, "g"), mv.cells_xml(conn, off, [12] * len(hexes)), len(p), len(hexes)))
    ctx = hr.Context(0)
    ctx.load_vtu(str(path))
    ctx.build_bvh()
    assert ctx.get_scene()["corners"].shape[0] == len(hexes)
    return ctx, oracle.OracleScene(scene_arrays_from_ctx(ctx))


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_vtu_scene_matches_oracle(vtu_scene, oracle, mode):
    ctx, osc = vtu_scene
    cam = hr.Camera((1.5, 1.2, 1.25), (0.5, 0.4, 0.33), vfov_deg=45.0)
    W, H = 160, 120
    rays = oracle.camera_rays(cam.lookfrom, cam.lookat, cam.vup, cam.vfov_deg, W, H)
    ctx.set_mode(hr.MODE_PLAIN if mode == "plain" else hr.MODE_BATCHED)
    h = ctx.intersect(rays, 0.0, False)
    _, hits = ctx.render(cam, [0.0], W, H, iso_zero_disables=True, want_rgb=False, want_hits=True)
    ctx.set_mode(hr.MODE_BATCHED)
    ref, _ = osc.trace(rays, 0.0, False, precision=64)
    assert (ref["kind"] == hr.HIT_FACE).mean() > 0.3
    box = ctx.boxes()
    h_elem = float(np.median((box[:, 3:] - box[:, :3]).max(1))) / 1.3  # padded box extent -> element size

    def trace(r):
        ctx.set_mode(hr.MODE_PLAIN if mode == "plain" else hr.MODE_BATCHED)
        return ctx.intersect(r, 0.0, False)

    parity.check_against_oracle(h, rays, osc, 0.0, False, h_elem, product_trace=trace, label=f"vtu {mode}")
    ctx.set_mode(hr.MODE_BATCHED)
    # ho_render makes its rays on the device, which may round a ray's
    # direction differently from the host's: compare with the oracle as well
    assert classify(hits[0].reshape(-1), ref).mean() >= 0.99
    assert (h["kind"] != hr.HIT_ISO).all()
