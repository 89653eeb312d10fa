"""ho_intersect_device_noalloc — the entry point for callers that may not
call the CUDA allocator while querying (an application whose own pool owns
all device memory, or a real-time loop that cannot absorb cudaFree's
device-wide synchronisation). Its scratch is a fixed device array for at most
HO_NOALLOC_MAX_RAYS rays per call.

Checked through the C ABI against the regular entry point, on two calls in a
row, with the FP64 check and polish of the regular entry point turned off
(this entry point returns the solvers' own answers): hit identity on >= 99.9%
of rays, t within 2e-4; the second call takes no device memory; a call over the
limit is refused with HO_ERR_RANGE; no ray reports an incomplete tree walk.
A second case puts prisms, quads and triangles beside the hexahedra, so the
call's primitive pass runs after its hexahedron kernels. This file sorts last
so a run that stops at the first failure has already run every other test.
"""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import oracle_bind as ob

pytestmark = pytest.mark.gpu


def _hits(buf):
    return buf.cpu().numpy().view(hr.HIT_DTYPE).reshape(-1)


def test_noalloc_matches_regular_entry_point_on_two_calls():
    import torch

    ctx, w = hr.workload_context("hex4_p4")
    W = H = 128  # 16,384 rays, under the per-call limit
    rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, W, H)
    n = rays.shape[0]
    iso = w.isovalues[0]
    ctx.set_mode(hr.MODE_BATCHED)
    ctx.set_option(hr.OPT_FP64_CHECK, 0)  # this entry point returns the solvers' own answers
    ref = ctx.intersect(rays, iso, True)
    ctx.set_option(hr.OPT_FP64_CHECK, 1)  # the existing entry point
    d_rays = torch.from_numpy(rays).cuda()
    d_out = torch.zeros(n * hr.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    free = []
    for call in range(2):
        d_out.fill_(0xFF)  # stale contents must not leak into the result
        ctx.intersect_device_noalloc(n, d_rays.data_ptr(), iso, True, d_out.data_ptr(), stream)
        torch.cuda.synchronize()
        got = _hits(d_out)
        same = (got["kind"] == ref["kind"]) & (got["elem"] == ref["elem"]) & (got["face"] == ref["face"])
        assert same.mean() >= 0.999, (call, same.mean())
        hit = same & (ref["kind"] > 0)
        assert np.abs(got["t"][hit] - ref["t"][hit]).max() < 2e-4, call
        assert (ref["kind"] > 0).sum() > 1000
        assert not (got["flags"] & hr.FLAG_INCOMPLETE).any()
        free.append(torch.cuda.mem_get_info()[0])
    # the first call places the fixed scratch array on the device (CUDA loads
    # module data lazily); after that a call takes no device memory
    assert abs(free[1] - free[0]) < (1 << 20)
    with pytest.raises(hr.HoError) as ei:
        ctx.intersect_device_noalloc(hr.NOALLOC_MAX_RAYS + 1, d_rays.data_ptr(), iso, True, d_out.data_ptr(), stream)
    assert ei.value.code == -7 and "limit" in str(ei.value)
    ctx.close()


def test_noalloc_hexahedra_with_primitives():
    """Hexahedra in [0, 1]^3 beside prisms, quads and triangles shifted to x
    in [1.1, 2.1]: the no-alloc call's hexahedron kernels, then its primitive
    pass, against the regular entry point."""
    import torch
    import prim_scenes

    from conftest import GOLDEN

    z = np.load(GOLDEN / "prims_ref.npz")
    arrs = ob.PrimArrays(z["kind"], z["verts"], z["geom_modes"], z["geom_offset"], z["geom"], z["field_modes"],
                         z["field_offset"], z["field"])
    ctx, w = hr.workload_context("hex4_p4", build=False)
    ctx.add_prim_arrays(prim_scenes.shifted(arrs, 1.1))
    ctx.build_bvh()
    ctx.set_mode(hr.MODE_BATCHED)
    cam = hr.Camera((1.05, 1.6, 3.2), (1.05, 0.3, 0.5), vfov_deg=55.0)
    rays = ob.camera_rays(cam.lookfrom, cam.lookat, cam.vup, cam.vfov_deg, 120, 90)
    n = rays.shape[0]
    iso = w.isovalues[0]
    ctx.set_option(hr.OPT_FP64_CHECK, 0)  # this entry point returns the solvers' own answers
    ref = ctx.intersect(rays, iso, True)
    ctx.set_option(hr.OPT_FP64_CHECK, 1)
    assert (ref["kind"] >= hr.HIT_PRISM).sum() > 100 and (ref["kind"] == hr.HIT_FACE).sum() > 100
    d_rays = torch.from_numpy(rays).cuda()
    d_out = torch.zeros(n * hr.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        d_out.fill_(0xFF)
        ctx.intersect_device_noalloc(n, d_rays.data_ptr(), iso, True, d_out.data_ptr(), stream)
        torch.cuda.synchronize()
        got = _hits(d_out)
        same = (got["kind"] == ref["kind"]) & (got["elem"] == ref["elem"]) & (got["face"] == ref["face"])
        assert same.mean() >= 0.999, (call, same.mean())
        hit = same & (ref["kind"] > 0)
        assert np.abs(got["t"][hit] - ref["t"][hit]).max() < 2e-4, call
        assert not (got["flags"] & hr.FLAG_INCOMPLETE).any()
    ctx.close()
