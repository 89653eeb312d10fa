"""Prisms, quads and curved triangles on the CPU: the oracle's restatement
of the reference's per-primitive code pinned against the reference itself,
and the C ABI's scene input.

Pinning: golden/prims_ref.npz (make_prims.py) holds the reference's own
boxes and IntersectRayWith* answers for 56 primitives (linear and curved,
all three kinds) and 2688 rays on given segments. The FP32 oracle must match
them bit for bit (boxes, hit or not, t, r, s, t-coordinate); where the
reference library is built here the same is checked live on a second scene.
"""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import oracle_bind as ob
import prim_scenes as ps
from conftest import GOLDEN

Z = np.load(GOLDEN / "prims_ref.npz")


def golden_arrays():
    return ob.PrimArrays(Z["kind"], Z["verts"], Z["geom_modes"], Z["geom_offset"], Z["geom"], Z["field_modes"],
                         Z["field_offset"], Z["field"])


def test_oracle_matches_reference_golden(oracle):
    arrs = golden_arrays()
    op = oracle.OraclePrims(arrs)
    assert np.array_equal(op.boxes(32), Z["ref_boxes"].astype(np.float64))
    rays, seg, owner, ref = Z["rays"], Z["seg"], Z["owner"], Z["ref_out"]
    hits = 0
    for p in range(arrs.n):
        m = owner == p
        mine = op.intersect(p, rays[m], seg[m], 32)
        assert np.array_equal(mine, ref[m]), (p, int(arrs.kind[p]))
        hits += int(mine[:, 0].sum())
    assert hits == int((ref[:, 0] > 0).sum()) > 1000
    # every kind hit, linear and curved
    for k in range(3):
        for curved in (False, True):
            sel = (arrs.kind[owner] == k) & ((arrs.geom_offset[owner] >= 0) == curved)
            assert (ref[sel, 0] > 0).sum() > 10, (k, curved)


@pytest.mark.skipif(not ob.ref_available(), reason="reference library not built here")
def test_oracle_matches_reference_live(oracle):
    arrs = ps.mixed_scene(seed=7, n_side=3)
    op = oracle.OraclePrims(arrs)
    boxes = op.boxes(32)
    rays, seg, owner = ps.rays_at_boxes(arrs, boxes, 30, np.random.default_rng(9))
    for p in range(arrs.n):
        m = owner == p
        rb, rr = ob.ref_prim_intersect(arrs, p, rays[m], seg[m])
        assert np.array_equal(rb.astype(np.float64), boxes[p])
        assert np.array_equal(op.intersect(p, rays[m], seg[m], 32), rr), p


def test_fp64_oracle_agrees_with_fp32(oracle):
    """The FP64 restatement finds a hit on the same rays almost always and,
    on nearly all rays both hit, the same root to FP32 accuracy. (The start
    searches branch on exact values and a prism's Newton iteration accepts
    any point of the ray inside it, so a few rays land on another root.)"""
    arrs = golden_arrays()
    op = oracle.OraclePrims(arrs)
    rays, seg, owner = Z["rays"], Z["seg"], Z["owner"]
    same = total = both_n = close = 0
    for p in range(arrs.n):
        m = owner == p
        a, b = op.intersect(p, rays[m], seg[m], 32), op.intersect(p, rays[m], seg[m], 64)
        both = (a[:, 0] > 0) & (b[:, 0] > 0)
        same += int((a[:, 0] == b[:, 0]).sum())
        total += int(m.sum())
        both_n += int(both.sum())
        close += int((np.abs(a[both, 1] - b[both, 1]) < 2e-3).sum())
    assert same >= 0.97 * total
    assert close >= 0.97 * both_n


def test_add_and_get_round_trip():
    arrs = golden_arrays()
    with hr.Context(0) as ctx:
        ctx.add_prim_arrays(arrs)
        g = ctx.get_prims()
        info = ctx.info()
    assert [info["n_prisms"], info["n_quads"], info["n_tris"]] == np.bincount(arrs.kind, minlength=3).tolist()
    for k in ("kind", "verts", "geom_modes", "field_modes"):
        assert np.array_equal(g[k], getattr(arrs, k)), k
    for p in range(arrs.n):
        for src, dst, pool_a, pool_b, modes in (("geom_offset", "geom_offsets", arrs.geom, g["geom"], "geom_modes"),
                                                ("field_offset", "field_offsets", arrs.field, g["field"],
                                                 "field_modes")):
            a, b = int(getattr(arrs, src)[p]), int(g[dst][p])
            assert (a < 0) == (b < 0)
            if a >= 0:
                m = getattr(arrs, modes)[p]
                blk = ps.block_size(int(arrs.kind[p]), [int(v) for v in m])
                reps = 3 if src == "geom_offset" else 1
                assert np.array_equal(pool_a[a:a + reps * blk], pool_b[b:b + reps * blk])


def test_insertion_order_within_kind():
    """Kinds may be added in any order; each kind keeps its own order and
    the list comes back prisms, quads, triangles."""
    tri = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32)
    quad = np.array([[[0, 0, 1], [1, 0, 1], [0, 1, 1], [1, 1, 1]]], np.float32)
    with hr.Context(0) as ctx:
        none2 = np.zeros((1, 2), np.uint32)
        neg = np.full(1, -1, np.int64)
        ctx.add_tris(tri, none2, np.zeros(0), neg, none2, np.zeros(0), neg)
        ctx.add_quads(quad, none2, np.zeros(0), neg, none2, np.zeros(0), neg)
        ctx.add_tris(tri + 2, none2, np.zeros(0), neg, none2, np.zeros(0), neg)
        g = ctx.get_prims()
    assert g["kind"].tolist() == [1, 2, 2]
    assert np.array_equal(g["verts"][1, :3], tri[0]) and np.array_equal(g["verts"][2, :3], tri[0] + 2)


@pytest.mark.parametrize("case", ["modes", "range", "field_range", "null"])
def test_argument_checks_leave_scene_unchanged(case):
    verts = np.zeros((1, 4, 3), np.float32)
    gm = np.array([[3, 3]], np.uint32)
    geom = np.zeros(27, np.float32)
    go = np.zeros(1, np.int64)
    fm = np.array([[2, 2]], np.uint32)
    field = np.zeros(4, np.float32)
    fo = np.zeros(1, np.int64)
    if case == "modes":
        gm[0, 0] = 10
        code = -7
    elif case == "range":
        geom = np.zeros(26, np.float32)
        code = -1
    elif case == "field_range":
        fo[0] = 1
        code = -1
    with hr.Context(0) as ctx:
        if case == "null":
            assert hr.lib.ho_add_quads(ctx.h, 1, None, None, None, 0, None, None, None, 0, None) == -1
        else:
            with pytest.raises(hr.HoError) as ei:
                ctx.add_quads(verts, gm, geom, go, fm, field, fo)
            assert ei.value.code == code
        assert ctx.get_prims()["kind"].size == 0
        gm_ok = np.array([[3, 3]], np.uint32)
        ctx.add_quads(verts, gm_ok, np.zeros(27, np.float32), np.zeros(1, np.int64), fm, np.zeros(4, np.float32),
                      np.zeros(1, np.int64))
        assert ctx.get_prims()["kind"].tolist() == [1]
