"""Generates the golden fixtures in this directory from the reference's own
host code (oracle/_ref/libref.so, built from the reference sources by
oracle/build_ref.sh). Run in a checkout that has the reference sources:

    python tests/golden/make_golden.py

Fixtures (all outputs are the reference's, computed in FP32 by its code):
  curvedface.npz  the reference loader's arrays for its single curved P=4 hex
                  sample (Hex_CurvedFace) and known answers on it: face hits,
                  isosurface roots, traced rays.
  hex4_p4.npz     the seeded hex4_p4 scene (4^3 hexes, P=4) + element-level
                  known answers (boxes, map, Jacobian/field/gradient, inverse
                  map, isosurface search, face search) + 4096 traced camera
                  rays with the reference's own candidate visit order.
  hex8_p6.npz     checksum of a seeded 8^3, P=6 scene (curving 0.08 h, 64
                  Gaussians, seed 2); 2048 traced rays, isovalues +-0.3.
  hex32_p6.npz    checksum of the seeded hex32_p6 scene (too large to store)
                  + 4096 rays through its cube traced at each isovalue
                  (-0.3, 0.0, 0.3; 0.0 with FindIsosurfaceOnRayHex called,
                  which the renderer skips at 0), with the visit order.
  hex64_p5.npz    the same for hex64_p5 (64^3 hexes, P=5, iso 0.1), 2048
                  rays.
"""
from __future__ import annotations

import hashlib
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "test-_gb300"))

import oracle_bind as ob  # noqa: E402
import workloads as hr  # noqa: E402  (workload definitions; no product library)

# The reference checkout is named by HORENDER_REFERENCE (its project root);
# the fixtures that need the reference's own files are skipped without it.
_REF_ROOT = os.environ.get("HORENDER_REFERENCE")
REF_DIR = Path(_REF_ROOT) / "FEM-AABB" if _REF_ROOT else None
ORDER_CAP = 32


def scene_arrays(name=None, **synth):
    """A workload's scene from the oracle's generator (the same arrays the
    product's ho_generate_synthetic makes; the tests check the digest)."""
    if name:
        synth = hr.WORKLOADS[name].synth()
    return ob.synth_scene(**synth)


def digest(arrs: ob.SceneArrays) -> str:
    h = hashlib.sha256()
    for a in (arrs.geom_modes, arrs.geom_offset, arrs.geom, arrs.field_modes, arrs.field_offset, arrs.field,
              arrs.verts):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def trace_fixture(rs: ob.RefScene, rays, iso):
    res, order, cnt = rs.trace(rays, iso, order_cap=ORDER_CAP)
    assert cnt.max() <= ORDER_CAP
    return res, order, cnt


def scene_payload(arrs: ob.SceneArrays, prefix="scene_"):
    return {prefix + k: getattr(arrs, k) for k in ("geom_modes", "geom_offset", "geom", "field_modes",
                                                     "field_offset", "field", "verts")}


def make_curvedface():
    if REF_DIR is None:
        sys.exit("set HORENDER_REFERENCE to the reference checkout to remake the curved-face fixture")
    rs = ob.RefScene(xml=str(REF_DIR / "Hex_CurvedFace.xml"), fld=str(REF_DIR / "Hex_CurvedFace.fld"))
    arrs = rs.arrays()
    rng = np.random.default_rng(101)
    # rays from all sides through the unit cube, plus the documented +z ray
    n = 512
    tgt = rng.uniform(0.05, 0.95, (n, 3))
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    orig = tgt - 2.5 * dirs
    rays = np.concatenate([orig, dirs], 1).astype(np.float32)
    rays[0] = [0.5, 0.5, -1.0, 0.0, 0.0, 1.0]
    seg = np.tile(np.array([0.001, 1e30], np.float32), (n, 1))
    hit = rs.hit_hex(0, rays, seg)
    iso_seg = np.tile(np.array([1.0, 2.0], np.float32), (1, 1))
    kat_iso = np.stack([rs.find_iso(0, rays[:1], iso_seg, v)[0] for v in (0.1, 0.3)])
    tr02, ord02, cnt02 = trace_fixture(rs, rays, 0.2)
    tr00, ord00, cnt00 = trace_fixture(rs, rays, 0.0)
    np.savez_compressed(HERE / "curvedface.npz", **scene_payload(arrs), rays=rays, hit_hex=hit, kat_iso=kat_iso,
                        trace_iso02=tr02, order_iso02=ord02, count_iso02=cnt02, trace_iso00=tr00,
                        order_iso00=ord00, count_iso00=cnt00)
    print("curvedface: face hit of the +z ray", hit[0], "iso KAT", kat_iso[:, :2])


def element_kats(rs: ob.RefScene, arrs, rng, elems):
    out = {}
    boxes4 = np.stack([rs.box(e, 4) for e in range(arrs.n)])
    boxes6 = np.stack([rs.box(e, 6) for e in range(arrs.n)])
    out["boxes4"], out["boxes6"] = boxes4, boxes6
    xi = rng.uniform(-1.2, 1.2, (len(elems), 128, 3)).astype(np.float32)
    out["kat_elems"] = np.array(elems, np.int32)
    out["kat_xi"] = xi
    out["kat_map"] = np.stack([rs.map_point(e, xi[i]) for i, e in enumerate(elems)])
    out["kat_eval"] = np.stack([rs.eval_point(e, xi[i]) for i, e in enumerate(elems)])
    pts = np.stack([rs.map_point(e, rng.uniform(-1, 1, (128, 3)).astype(np.float32)) for e in elems])
    out["kat_inv_x"] = pts
    out["kat_inv"] = np.stack([rs.inverse_map(e, pts[i]) for i, e in enumerate(elems)])
    # rays through each element's box, iso search on its box segment, face search
    rays_all, segs_all = [], []
    for e in elems:
        lo, hi = boxes4[e, :3], boxes4[e, 3:]
        c = 0.5 * (lo + hi)
        tgt = c + (hi - lo) * rng.uniform(-0.35, 0.35, (128, 3))
        d = rng.normal(size=(128, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        o = tgt - 1.5 * d
        rays = np.concatenate([o, d], 1).astype(np.float32)
        rays_all.append(rays)
        segs_all.append(np.tile(np.array([0.001, 1e30], np.float32), (128, 1)))
    rays_all = np.stack(rays_all)
    out["kat_rays"] = rays_all
    out["kat_hit_hex"] = np.stack([rs.hit_hex(e, rays_all[i], segs_all[i]) for i, e in enumerate(elems)])
    # iso on the (reference-computed) box segment of each ray
    iso_seg = np.zeros((len(elems), 128, 2), np.float32)
    for i, e in enumerate(elems):
        lo, hi = boxes4[e, :3].astype(np.float64), boxes4[e, 3:].astype(np.float64)
        o, d = rays_all[i, :, :3].astype(np.float64), rays_all[i, :, 3:].astype(np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            t0 = (lo - o) / d
            t1 = (hi - o) / d
        te = np.maximum(np.minimum(t0, t1).max(1), 0.001)
        tx = np.maximum(t0, t1).min(1)
        iso_seg[i, :, 0], iso_seg[i, :, 1] = te, tx
    out["kat_iso_seg"] = iso_seg
    out["kat_isovalue"] = np.float32(0.1)
    out["kat_find_iso"] = np.stack([rs.find_iso(e, rays_all[i], iso_seg[i], 0.1) for i, e in enumerate(elems)])
    return out


def make_hex4():
    arrs = scene_arrays("hex4_p4")
    rs = ob.RefScene(arrs)
    rng = np.random.default_rng(202)
    kats = element_kats(rs, arrs, rng, [0, 21, 42, 63])
    w = hr.WORKLOADS["hex4_p4"]
    rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, w.width, w.height)
    sub = rays[::16].copy()
    tr, order, cnt = trace_fixture(rs, sub, 0.2)
    tr0, order0, cnt0 = trace_fixture(rs, sub, 0.0)
    np.savez_compressed(HERE / "hex4_p4.npz", **scene_payload(arrs), **kats, rays=sub, trace_iso=tr,
                        order_iso=order, count_iso=cnt, trace_faces=tr0, order_faces=order0, count_faces=cnt0,
                        isovalue=np.float32(0.2))
    print("hex4_p4: traced", sub.shape[0], "rays; kinds", np.bincount(tr[:, 0].astype(int), minlength=3))


def make_hex8():
    synth = dict(nx=8, ny=8, nz=8, order_min=6, order_max=6, curve_amp=0.08, n_gauss=64, seed=2)
    arrs = scene_arrays(**synth)
    rs = ob.RefScene(arrs)
    w = hr.WORKLOADS["hex32_p6"]
    rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, 480, 270)
    rng = np.random.default_rng(303)
    sub = rays[rng.choice(rays.shape[0], 2048, replace=False)]
    payload = {}
    for tag, iso in (("m03", -0.3), ("p03", 0.3)):
        tr, order, cnt = trace_fixture(rs, sub, iso)
        payload[f"trace_{tag}"], payload[f"order_{tag}"], payload[f"count_{tag}"] = tr, order, cnt
    np.savez_compressed(HERE / "hex8_p6.npz", digest=np.array(digest(arrs)), rays=sub, **payload)
    print("hex8_p6: kinds", np.bincount(payload["trace_p03"][:, 0].astype(int), minlength=3))


def scene_box_rays(w, n, seed):
    """n of the workload's pixel-centre rays that meet the scene box (the
    others are trivially misses), drawn without replacement."""
    rays = ob.camera_rays(w.camera.lookfrom, w.camera.lookat, w.camera.vup, w.camera.vfov_deg, w.width, w.height)
    o, d = rays[:, :3].astype(np.float64), rays[:, 3:].astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        t0 = (-0.01 - o) / d
        t1 = (1.01 - o) / d
    te = np.minimum(t0, t1).max(1)
    tx = np.maximum(t0, t1).min(1)
    inside = np.where(tx > te)[0]
    rng = np.random.default_rng(seed)
    return rays[np.sort(rng.choice(inside, n, replace=False))]


def iso_tag(iso):
    return ("m" if iso < 0 else "p") + f"{abs(iso):.1f}".replace(".", "")


def make_workload_fixture(name, n_rays, seed, out):
    """The reference's traces of n_rays rays at every isovalue of a workload,
    with its visit order. Isovalue 0.0 is traced with the isosurface on
    (FindIsosurfaceOnRayHex called at 0.0; the renderer would turn it off)."""
    w = hr.WORKLOADS[name]
    arrs = scene_arrays(name)
    sub = scene_box_rays(w, n_rays, seed)
    rs = ob.RefScene(arrs)
    payload = {}
    for iso in w.isovalues:
        tag = iso_tag(iso)
        tr, order, cnt = rs.trace(sub, iso, order_cap=ORDER_CAP, iso_always=True)
        assert cnt.max() <= ORDER_CAP, cnt.max()
        payload[f"trace_{tag}"], payload[f"order_{tag}"], payload[f"count_{tag}"] = tr, order, cnt
        print(f"{name} iso {iso}: kinds {np.bincount(tr[:, 0].astype(int), minlength=3)}, most candidates {cnt.max()}",
              flush=True)
    np.savez_compressed(HERE / out, digest=np.array(digest(arrs)), rays=sub,
                        isovalues=np.asarray(w.isovalues, np.float32), **payload)


def make_hex32():
    make_workload_fixture("hex32_p6", 4096, 404, "hex32_p6.npz")


def make_hex64():
    make_workload_fixture("hex64_p5", 2048, 505, "hex64_p5.npz")


if __name__ == "__main__":
    if not ob.ref_available():
        sys.exit("oracle/_ref/libref.so is missing: run oracle/build_ref.sh in a checkout with the reference")
    which = sys.argv[1:] or ["curvedface", "hex4", "hex8", "hex32", "hex64"]
    for w in which:
        globals()[f"make_{w}"]()
