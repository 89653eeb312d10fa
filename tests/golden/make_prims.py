"""Generates tests/golden/prims_ref.npz: a seeded scene of prisms, quads and
curved triangles (tests/prim_scenes.py, linear and curved, most with a
field), rays aimed at each primitive's box with segments [0.001, tmax], and
what the reference's own code makes of them (FEM-AABB/fem/PrismElement.cu,
QuadElement.cu, TriElement.cu through oracle/_ref/libref.so): every
primitive's sampled box and, per ray, IntersectRayWith*'s answer (hit, t,
r, s, t-coordinate).

Run: python tests/golden/make_prims.py (needs oracle/_ref/libref.so).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1] / "test-_gb300"))


def main():
    import oracle_bind as ob
    import prim_scenes as ps

    if not ob.ref_available():
        sys.exit("oracle/_ref/libref.so not built (oracle/build_ref.sh)")
    arrs = ps.mixed_scene(seed=1)
    boxes = ob.OraclePrims(arrs).boxes(32)
    rays, seg, owner = ps.rays_at_boxes(arrs, boxes, 48, np.random.default_rng(4))
    ref_boxes = np.zeros((arrs.n, 6), np.float32)
    ref_out = np.zeros((rays.shape[0], 5))
    for p in range(arrs.n):
        m = owner == p
        ref_boxes[p], ref_out[m] = ob.ref_prim_intersect(arrs, p, rays[m], seg[m])
    np.savez_compressed(HERE / "prims_ref.npz", kind=arrs.kind, verts=arrs.verts, geom_modes=arrs.geom_modes,
                        geom_offset=arrs.geom_offset, geom=arrs.geom, field_modes=arrs.field_modes,
                        field_offset=arrs.field_offset, field=arrs.field, rays=rays, seg=seg, owner=owner,
                        ref_boxes=ref_boxes, ref_out=ref_out)
    hits = ref_out[:, 0] > 0
    print(f"{arrs.n} primitives, {rays.shape[0]} rays, {int(hits.sum())} reference hits")


if __name__ == "__main__":
    main()
