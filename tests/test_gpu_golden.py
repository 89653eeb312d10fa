"""GPU kernels against the reference's own traced rays (golden fixtures made
from the reference build) and against the oracle, through the C ABI.

Per ray the GPU answer (kind, element, face) must equal the reference's,
except on rays where the reference's answer depends on its BVH visit order
(the oracle's ascending-entry order gives a different answer there too,
and the fixture's recorded reference order reproduces the reference's);
those rays are counted, not failed. Against the ordered oracle the GPU must
agree on >= 99.5% of rays, or all but 2 on small samples (the rest are FP32
near-ties, counted), with t
within 2e-4 where the identities agree.
"""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import oracle_bind as ob
from conftest import GOLDEN, scene_arrays_from_ctx

pytestmark = pytest.mark.gpu


def _ctx_for(synth):
    ctx = hr.Context(0)
    ctx.generate_synthetic(**synth)
    ctx.build_bvh()
    return ctx


def _compare(ctx, osc, rays, iso, ref_tr, label):
    g = ctx.intersect(rays, iso, iso != 0.0)
    o, _ = osc.trace(rays, iso, iso != 0.0, precision=32)
    rk, re_, rf = ref_tr[:, 0].astype(int), ref_tr[:, 1].astype(int), ref_tr[:, 2].astype(int)
    g_ref = (g["kind"] == rk) & (g["elem"] == re_) & (g["face"] == rf)
    o_ref = (o["kind"] == rk) & (o["elem"] == re_) & (o["face"] == rf)
    g_o = (g["kind"] == o["kind"]) & (g["elem"] == o["elem"]) & (g["face"] == o["face"])
    order_dep = ~o_ref
    unexplained = ~g_ref & ~order_dep
    print(f"{label}: rays {rays.shape[0]}, gpu==ref {g_ref.mean():.4f}, order-dependent {order_dep.sum()}, "
          f"gpu!=ref otherwise {unexplained.sum()}, gpu==oracle {g_o.mean():.4f}")
    n = rays.shape[0]
    allowed = max(2, int(0.005 * n))  # FP32 near-ties (sample-size floor of 2 rays)
    assert (~g_o).sum() <= allowed
    assert unexplained.sum() <= allowed
    m = g_ref & (rk > 0)
    if m.any():
        assert np.abs(g["t"][m] - ref_tr[m, 3]).max() < 2e-4
    return g, o


def test_hex4_against_reference():
    z = np.load(GOLDEN / "hex4_p4.npz")
    ctx = _ctx_for(hr.WORKLOADS["hex4_p4"].synth())
    osc = ob.OracleScene(scene_arrays_from_ctx(ctx))
    _compare(ctx, osc, z["rays"], float(z["isovalue"]), z["trace_iso"], "hex4 iso 0.2")
    _compare(ctx, osc, z["rays"], 0.0, z["trace_faces"], "hex4 faces")


def test_hex8_against_reference():
    z = np.load(GOLDEN / "hex8_p6.npz")
    ctx = _ctx_for(dict(nx=8, ny=8, nz=8, order_min=6, order_max=6, curve_amp=0.08, n_gauss=64, seed=2))
    osc = ob.OracleScene(scene_arrays_from_ctx(ctx))
    for tag, iso in (("m03", -0.3), ("p03", 0.3)):
        _compare(ctx, osc, z["rays"], iso, z[f"trace_{tag}"], f"hex8 iso {iso}")


def test_hex32_against_reference_and_fp64_error():
    z = np.load(GOLDEN / "hex32_p6.npz")
    ctx = _ctx_for(hr.WORKLOADS["hex32_p6"].synth())
    osc = ob.OracleScene(scene_arrays_from_ctx(ctx))
    for tag, iso in (("m03", -0.3), ("p03", 0.3)):
        g, o = _compare(ctx, osc, z["rays"], iso, z[f"trace_{tag}"], f"hex32 iso {iso}")
        o64, _ = osc.trace(z["rays"], iso, True, precision=64)
        same = (g["kind"] == o64["kind"]) & (g["elem"] == o64["elem"]) & (g["face"] == o64["face"]) & (
            g["kind"] > 0)
        err = np.abs(g["t"][same] - o64["t"][same])
        print(f"hex32 iso {iso}: |t_gpu - t_fp64| max {err.max():.2e} median {np.median(err):.2e}")
        assert err.max() < 2e-4
