"""The oracle pinned against the reference's own host code (golden fixtures
made by tests/golden/make_golden.py from the reference build).

* Element functions: the oracle's FP32 instantiation reproduces the
  reference bit for bit (same steps, same rounding).
* Traversal: replaying the reference's own candidate visit order through the
  oracle reproduces every traced ray bit for bit; the oracle's ordered
  candidate policy (ascending box entry) agrees with the reference's BVH-order
  result on >= 99.5% of rays, and every ray where they differ is one whose
  answer depends on visit order (the replay reproduces the reference there).
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import oracle_bind as ob
from conftest import GOLDEN


def _scene(z, prefix="scene_"):
    return ob.SceneArrays(z[prefix + "geom_modes"], z[prefix + "geom_offset"], z[prefix + "geom"],
                          z[prefix + "field_modes"], z[prefix + "field_offset"], z[prefix + "field"],
                          z[prefix + "verts"])


def _digest(arrs):
    h = hashlib.sha256()
    for a in (arrs.geom_modes, arrs.geom_offset, arrs.geom, arrs.field_modes, arrs.field_offset, arrs.field,
              arrs.verts):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _synth_arrays(**synth):
    import horender as hr

    ctx = hr.Context(0)
    ctx.generate_synthetic(**synth)
    s = ctx.get_scene()
    ctx.close()
    return ob.SceneArrays(s["geom_modes"], s["geom_offsets"], s["geom"], s["field_modes"], s["field_offsets"],
                          s["field"], s["corners"])


def _ref_ids(tr):
    return tr[:, 0].astype(int), tr[:, 1].astype(int), tr[:, 2].astype(int)


def _check_replay_bit_exact(osc, rays, iso, tr, order, cnt, iso_on=None):
    iso_on = iso != 0.0 if iso_on is None else iso_on
    rep = osc.trace_replay(rays, iso, iso_on, order, cnt, precision=32)
    k, e, f = _ref_ids(tr)
    assert np.array_equal(rep["kind"], k) and np.array_equal(rep["elem"], e) and np.array_equal(rep["face"], f)
    hit = k > 0
    assert np.array_equal(rep["t"][hit].astype(np.float32), tr[hit, 3])
    assert np.array_equal(rep["xi"][hit].astype(np.float32), tr[hit, 4:7])
    assert np.array_equal(rep["n"][hit].astype(np.float32), tr[hit, 7:10])


def _check_ordered_policy(osc, rays, iso, tr, order, cnt, min_agree=0.995, iso_on=None):
    iso_on = iso != 0.0 if iso_on is None else iso_on
    out, _ = osc.trace(rays, iso, iso_on, precision=32)
    k, e, f = _ref_ids(tr)
    same = (out["kind"] == k) & (out["elem"] == e) & (out["face"] == f)
    assert same.mean() >= min_agree, same.mean()
    # t agrees to the stopping tolerance where the ids agree; where the two
    # stopped further apart (the candidate's segment, clipped by a different
    # earlier hit, moved the scan samples), both are the same root: polished
    # to it, they agree
    hit = same & (k > 0)
    far = np.where(hit & (np.abs(out["t"] - tr[:, 3]) >= 2e-4))[0]
    assert far.size <= max(2, hit.sum() // 500), far.size
    if far.size:
        ref = np.zeros(far.size, ob.HIT_DTYPE)
        ref["kind"], ref["elem"], ref["face"] = k[far], e[far], f[far]
        ref["t"], ref["xi"] = tr[far, 3], tr[far, 4:7]
        p_ref = osc.polish(rays[far], ref, iso)
        p_out = osc.polish(rays[far], out[far], iso)
        assert (p_ref["pad"] == 1).all() and (p_out["pad"] == 1).all()
        assert np.abs(p_ref["t"] - p_out["t"]).max() < 1e-7
    # every disagreement is a visit-order effect: replaying the reference's
    # order through the same per-candidate policy gives the reference's answer
    bad = np.where(~same)[0]
    if bad.size:
        rep = osc.trace_replay(rays[bad], iso, iso_on, order[bad], cnt[bad], precision=32)
        assert np.array_equal(rep["kind"], k[bad]) and np.array_equal(rep["elem"], e[bad])
    return same


def test_curvedface_known_answers(oracle):
    z = np.load(GOLDEN / "curvedface.npz")
    osc = ob.OracleScene(_scene(z))
    rays = z["rays"]
    # the documented ray (0.5,0.5,-1) +z meets the curved face 0 at t = 0.7
    h = osc.hit_hex(0, rays[:1], [[0.001, 1e30]], precision=32)
    assert h[0, 0] == 1 and h[0, 5] == 0 and abs(h[0, 1] - 0.7) < 1e-6
    for j, v in enumerate((0.1, 0.3)):
        r = osc.find_iso(0, rays[:1], [[1.0, 2.0]], v, precision=32)
        assert r[0, 0] == 1 and np.float32(r[0, 1]) == z["kat_iso"][j, 1]
    hh = osc.hit_hex(0, rays, np.tile([0.001, 1e30], (rays.shape[0], 1)), precision=32).astype(np.float32)
    assert np.array_equal(hh, z["hit_hex"])


def test_curvedface_traces(oracle):
    z = np.load(GOLDEN / "curvedface.npz")
    osc = ob.OracleScene(_scene(z))
    for tag, iso in (("iso02", 0.2), ("iso00", 0.0)):
        _check_replay_bit_exact(osc, z["rays"], iso, z[f"trace_{tag}"], z[f"order_{tag}"], z[f"count_{tag}"])
        _check_ordered_policy(osc, z["rays"], iso, z[f"trace_{tag}"], z[f"order_{tag}"], z[f"count_{tag}"])


@pytest.fixture(scope="module")
def hex4(oracle):
    z = np.load(GOLDEN / "hex4_p4.npz")
    return z, ob.OracleScene(_scene(z))


def test_generator_reproduces_hex4_fixture(hex4):
    import horender as hr

    z, _ = hex4
    arrs = _synth_arrays(**hr.WORKLOADS["hex4_p4"].synth())
    ref = _scene(z)
    for k in ("geom_modes", "geom_offset", "geom", "field_modes", "field_offset", "field", "verts"):
        assert np.array_equal(getattr(arrs, k), getattr(ref, k)), k


def test_hex4_boxes_bit_exact(hex4):
    z, osc = hex4
    assert np.array_equal(osc.boxes(32).astype(np.float32), z["boxes4"])


def test_hex4_element_functions_bit_exact(hex4):
    z, osc = hex4
    for i, e in enumerate(z["kat_elems"]):
        xi = z["kat_xi"][i].astype(np.float64)
        assert np.array_equal(osc.map_point(e, xi, 32).astype(np.float32), z["kat_map"][i])
        assert np.array_equal(osc.eval_point(e, xi, 32).astype(np.float32), z["kat_eval"][i])
        assert np.array_equal(osc.inverse_map(e, z["kat_inv_x"][i], 32).astype(np.float32), z["kat_inv"][i])
        seg = np.tile([0.001, 1e30], (z["kat_rays"].shape[1], 1))
        assert np.array_equal(osc.hit_hex(e, z["kat_rays"][i], seg, 32).astype(np.float32), z["kat_hit_hex"][i])
        fi = osc.find_iso(e, z["kat_rays"][i], z["kat_iso_seg"][i], float(z["kat_isovalue"]), 32)
        assert np.array_equal(fi.astype(np.float32), z["kat_find_iso"][i])


def test_hex4_traces(hex4):
    z, osc = hex4
    iso = float(z["isovalue"])
    _check_replay_bit_exact(osc, z["rays"], iso, z["trace_iso"], z["order_iso"], z["count_iso"])
    _check_replay_bit_exact(osc, z["rays"], 0.0, z["trace_faces"], z["order_faces"], z["count_faces"])
    _check_ordered_policy(osc, z["rays"], iso, z["trace_iso"], z["order_iso"], z["count_iso"])
    _check_ordered_policy(osc, z["rays"], 0.0, z["trace_faces"], z["order_faces"], z["count_faces"])


def test_hex4_fp64_oracle_agrees_with_fp32(hex4):
    z, osc = hex4
    a, _ = osc.trace(z["rays"], 0.2, True, precision=32)
    b, _ = osc.trace(z["rays"], 0.2, True, precision=64)
    same = (a["kind"] == b["kind"]) & (a["elem"] == b["elem"]) & (a["face"] == b["face"])
    assert same.mean() >= 0.999
    hit = same & (a["kind"] > 0)
    assert np.abs(a["t"][hit] - b["t"][hit]).max() < 1e-4


@pytest.mark.parametrize("name,synth", [
    ("hex8_p6.npz", dict(nx=8, ny=8, nz=8, order_min=6, order_max=6, curve_amp=0.08, n_gauss=64, seed=2)),
])
def test_hex8_traces(oracle, name, synth):
    z = np.load(GOLDEN / name)
    arrs = _synth_arrays(**synth)
    assert _digest(arrs) == str(z["digest"])
    osc = ob.OracleScene(arrs)
    for tag, iso in (("m03", -0.3), ("p03", 0.3)):
        _check_replay_bit_exact(osc, z["rays"], iso, z[f"trace_{tag}"], z[f"order_{tag}"], z[f"count_{tag}"])
        _check_ordered_policy(osc, z["rays"], iso, z[f"trace_{tag}"], z[f"order_{tag}"], z[f"count_{tag}"])


@pytest.mark.parametrize("name", ["hex32_p6", "hex64_p5"])
def test_workload_traces(oracle, name):
    """The benchmark workloads' fixtures (4096 / 2048 rays through the cube at
    every isovalue, 0.0 with the isosurface on): the scene from the oracle's
    generator has the fixture's digest; on the first 1024 rays, replaying the
    reference's visit order reproduces every traced ray bit for bit, and the
    product's ascending order agrees on at least 97% of rays with every
    disagreement the order (the lowest, hex32_p6 at iso 0.3, agrees on 97.6%
    of the 1024 rays)."""
    import workloads

    z = np.load(GOLDEN / f"{name}.npz")
    arrs = ob.synth_scene(**workloads.WORKLOADS[name].synth())
    assert _digest(arrs) == str(z["digest"])
    osc = ob.OracleScene(arrs)
    n = 1024  # of the fixture's rays (the GPU tests use all of them)
    for iso in [float(v) for v in z["isovalues"]]:
        tag = ("m" if iso < 0 else "p") + f"{abs(iso):.1f}".replace(".", "")
        args = (osc, z["rays"][:n], iso, z[f"trace_{tag}"][:n], z[f"order_{tag}"][:n], z[f"count_{tag}"][:n])
        _check_replay_bit_exact(*args, iso_on=True)
        _check_ordered_policy(*args, min_agree=0.97, iso_on=True)
