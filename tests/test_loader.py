"""Nektar++ XML/FLD loader (ho_load_xml_fld) against the reference loader.

The fixtures under golden/nektar are generated meshes (make_nektar.py) plus
the arrays the reference's own loader made of them. Criteria:
  * element count and order, geometry/field modes, offsets, corner vertices
    and field coefficients: identical (the field is FP64 -> FP32 casts or
    FP32 text parses on both sides);
  * geometry: the reference builds it in mixed FP32/FP64, the product in
    FP64 from the same FP32 inputs, so mapped positions x(xi) agree within
    1e-6 on a 7^3 grid of reference points (domain size 1) and modal
    coefficients within 5e-5.
"""
from __future__ import annotations

import base64
import os
import zlib
from pathlib import Path

import numpy as np
import pytest

import horender as hr
from conftest import GOLDEN, scene_arrays_from_ctx

NEK = GOLDEN / "nektar"
CASES = ["nek_faces", "nek_verts", "nek_raw", "nek_fp32"]
# the reference's own sample mesh, read from the checkout HORENDER_REFERENCE names (skipped without it)
_REF_ROOT = os.environ.get("HORENDER_REFERENCE")
REF_SAMPLE = Path(_REF_ROOT) / "FEM-AABB" / "Hex_CurvedFace.xml" if _REF_ROOT else None


def load(name, fld=None):
    ctx = hr.Context(0)
    ctx.load_xml_fld(str(NEK / f"{name}.xml"), str(fld or NEK / f"{name}.fld"))
    return ctx


@pytest.mark.parametrize("name", CASES)
def test_matches_reference_loader(name, oracle):
    ref = np.load(NEK / f"{name}.npz")
    with load(name) as ctx:
        s = ctx.get_scene()
        mine = scene_arrays_from_ctx(ctx)
    assert np.array_equal(s["geom_modes"], ref["geom_modes"])
    assert np.array_equal(s["field_modes"], ref["field_modes"])
    assert np.array_equal(s["geom_offsets"], ref["geom_offset"])
    assert np.array_equal(s["field_offsets"], ref["field_offset"])
    assert np.array_equal(s["corners"], ref["verts"])
    assert np.array_equal(s["field"], ref["field"][: s["field"].size])
    assert np.abs(s["geom"] - ref["geom"][: s["geom"].size]).max() < 5e-5
    theirs = oracle.SceneArrays(ref["geom_modes"], ref["geom_offset"], ref["geom"], ref["field_modes"],
                                ref["field_offset"], ref["field"], ref["verts"])
    a, b = oracle.OracleScene(mine), oracle.OracleScene(theirs)
    g = np.linspace(-1.0, 1.0, 7)
    xi = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    for e in range(mine.n):
        assert np.abs(a.map_point(e, xi) - b.map_point(e, xi)).max() < 1e-6, f"element {e}"


def test_curved_geometry_is_used():
    """nek_faces has curved edges and faces: its geometry is not trilinear."""
    with load("nek_faces") as ctx:
        s = ctx.get_scene()
    curved = 0
    for e, (m0, m1, m2) in enumerate(s["geom_modes"]):
        o = s["geom_offsets"][e]
        g = s["geom"][o:o + 3 * m0 * m1 * m2].reshape(3, m2, m1, m0)
        lin = g[:, :2, :2, :2].copy()
        g[:, :2, :2, :2] = 0.0  # vertex modes; the rest is curvature
        curved += np.abs(g).max() > 1e-3
        assert np.abs(lin).max() > 0.0
    assert curved >= len(s["geom_modes"]) // 2


def test_vertex_zero_read_from_file():
    """The product reads vertex 0's coordinates from the file (the reference's
    vertex scan leaves vertex 0 at the origin)."""
    with load("nek_origin") as ctx:
        s = ctx.get_scene()
    assert np.allclose(s["corners"][0, 0], [2.0, -1.0, 0.5])
    assert np.allclose(s["corners"][0, 6], [3.0, 0.0, 1.5])


def _payloads(coef: np.ndarray):
    f8 = coef.astype("<f8").tobytes()
    raw = zlib.compressobj(6, zlib.DEFLATED, -15)
    yield "ascii", " ".join(f"{c:.9g}" for c in coef), np.float32([float(f"{c:.9g}") for c in coef])
    for level in (0, 1, 9):  # stored, fixed/dynamic Huffman
        yield f"zlib{level}", base64.b64encode(zlib.compress(f8, level)).decode(), coef.astype(np.float32)
    yield "deflate", base64.b64encode(raw.compress(f8) + raw.flush()).decode(), coef.astype(np.float32)
    yield "plain", base64.b64encode(f8).decode(), coef.astype(np.float32)


def test_payload_encodings(tmp_path):
    rng = np.random.default_rng(7)
    n = 2 * (4 * 120 + 4 * 27)  # nek_verts: 8 hexes, two fields
    coef = rng.standard_normal(n)
    for kind, payload, want in _payloads(coef):
        fld = tmp_path / f"{kind}.fld"
        fld.write_text(f'<NEKTAR>\n<ELEMENTS FIELDS="u,v">\n{payload}\n</ELEMENTS>\n</NEKTAR>\n')
        with load("nek_verts", fld) as ctx:
            s = ctx.get_scene()
        # field u of the 8 hexes: the first 4*120 + 4*27 values, in order
        assert np.array_equal(s["field"], want[: s["field"].size]), kind


def test_short_stream_leaves_rest_without_field(tmp_path):
    fld = tmp_path / "short.fld"
    fld.write_text('<ELEMENTS FIELDS="u,v">' + " ".join(["1.5"] * 250) + "</ELEMENTS>")
    with load("nek_verts", fld) as ctx:
        s = ctx.get_scene()
    # 4 hexes of 120 coefficients: two fit, the third would overrun
    assert s["field_offsets"].tolist()[:3] == [0, 120, -1]
    assert (s["field_offsets"][2:] == -1).all()


def test_missing_field_file_loads_geometry(tmp_path):
    with load("nek_raw", tmp_path / "absent.fld") as ctx:
        s = ctx.get_scene()
    assert s["geom_offsets"].shape[0] == 2 and (s["field_offsets"] == -1).all()


def test_errors_leave_scene_unchanged(tmp_path):
    with hr.Context(0) as ctx:
        ctx.load_xml_fld(str(NEK / "nek_raw.xml"), str(NEK / "nek_raw.fld"))
        with pytest.raises(hr.HoError) as ei:
            ctx.load_xml_fld(str(tmp_path / "absent.xml"), str(NEK / "nek_raw.fld"))
        assert ei.value.code == -4
        no_hex = tmp_path / "nohex.xml"
        no_hex.write_text('<NEKTAR><GEOMETRY><VERTEX><V ID="0"> 0 0 0 </V></VERTEX></GEOMETRY></NEKTAR>')
        with pytest.raises(hr.HoError) as ei:
            ctx.load_xml_fld(str(no_hex), str(NEK / "nek_raw.fld"))
        assert ei.value.code == -5
        big = tmp_path / "big.xml"
        big.write_text((NEK / "nek_raw.xml").read_text().replace('NUMMODES="6"', 'NUMMODES="12"'))
        with pytest.raises(hr.HoError) as ei:
            ctx.load_xml_fld(str(big), str(NEK / "nek_raw.fld"))
        assert ei.value.code == -7
        s = ctx.get_scene()
        assert s["geom_offsets"].shape[0] == 2


def test_load_appends_to_scene():
    with hr.Context(0) as ctx:
        ctx.load_xml_fld(str(NEK / "nek_raw.xml"), str(NEK / "nek_raw.fld"))
        ctx.load_xml_fld(str(NEK / "nek_fp32.xml"), str(NEK / "nek_fp32.fld"))
        s = ctx.get_scene()
    assert s["geom_offsets"].shape[0] == 5
    assert s["field_offsets"].tolist() == [0, 216, 432, 459, 486]


@pytest.mark.skipif(REF_SAMPLE is None or not REF_SAMPLE.exists(), reason="reference sample mesh not present")
def test_reference_sample_mesh():
    """The reference's own curved-face sample against the arrays its loader made."""
    g = np.load(GOLDEN / "curvedface.npz")
    with hr.Context(0) as ctx:
        ctx.load_xml_fld(str(REF_SAMPLE), str(REF_SAMPLE.with_suffix(".fld")))
        s = ctx.get_scene()
    assert np.array_equal(s["geom_modes"].reshape(-1), g["scene_geom_modes"].reshape(-1))
    assert np.array_equal(s["field"], g["scene_field"][: s["field"].size])
    assert np.abs(s["geom"] - g["scene_geom"][: s["geom"].size]).max() < 1e-5


@pytest.mark.gpu
def test_loaded_mesh_renders_like_oracle(oracle):
    """A loaded curved mesh through the GPU path against the FP64 oracle on
    the same loaded arrays (iso 0.3 on field u). This mesh is strongly bent,
    so some rays are precision-sensitive: the FP32 and FP64 oracles already
    disagree on about 0.6% of them (a sample near a bracket edge, or an
    inverse map outside the element that converges in one precision only).
    Every identity difference must be one of the classes of tests/parity.py
    (tie, grazing, or a ray at a decision boundary of the algorithm), and the
    agreeing hits' t, xi and u lie within the bounds of the FP64 judge."""
    import parity

    with load("nek_faces") as ctx:
        ctx.build_bvh()
        arrs = scene_arrays_from_ctx(ctx)
        osc = oracle.OracleScene(arrs)
        cam = hr.Camera((2.2, 1.7, 1.9), (0.5, 0.5, 0.5))
        W = H = 96
        _, hits = ctx.render(cam, [0.3], W, H, iso_zero_disables=True, want_rgb=False, want_hits=True)
        h = hits[0].reshape(-1)
        rays = oracle.camera_rays(cam.lookfrom, cam.lookat, cam.vup, cam.vfov_deg, W, H)
        box = ctx.boxes()
        h_elem = float(np.median((box[:, 3:] - box[:, :3]).max(1))) / 1.3  # padded box extent -> element size
        cnt = parity.check_against_oracle(h, rays, osc, 0.3, True, h_elem, label="loaded mesh",
                                          product_trace=lambda r: ctx.intersect(r, 0.3, True))
        assert cnt["differ"] <= 0.05 * h.size
