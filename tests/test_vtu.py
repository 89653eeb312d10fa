"""VTK XML unstructured-grid loader (ho_load_vtu) against the reference's
loader (load_vtu_file, FEM-AABB/vtu_loader.cpp:156-343).

The fixtures under golden/vtu and what the reference loader made of them
(vtu_ref.npz) come from make_vtu.py. Criteria: the same hexahedra, prisms
and quads, in the same order, with bit-identical vertices (both sides parse
the text as float); a file without any of those cells fails on both sides;
every failure leaves the scene unchanged."""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
from conftest import GOLDEN

VTU = GOLDEN / "vtu"
REF = np.load(VTU / "vtu_ref.npz")
CASES = ["grid", "mixed", "nooffsets", "badrange", "badindex", "wide", "nohex"]


@pytest.mark.parametrize("name", CASES)
def test_matches_reference_loader(name):
    assert bool(REF[f"{name}_ok"])
    with hr.Context(0) as ctx:
        ctx.load_vtu(str(VTU / f"{name}.vtu"))
        s = ctx.get_scene()
        p = ctx.get_prims()
    counts = REF[f"{name}_counts"]
    assert np.array_equal(np.bincount(p["kind"], minlength=3), [counts[1], counts[2], 0])
    assert np.array_equal(p["verts"][p["kind"] == 0], REF[f"{name}_prisms"])
    assert np.array_equal(p["verts"][p["kind"] == 1][:, :4], REF[f"{name}_quads"])
    assert (p["geom_offsets"] == -1).all() and (p["field_offsets"] == -1).all()
    ref_verts = REF[f"{name}_verts"]
    assert len(s["corners"]) == int(REF[f"{name}_counts"][0]) == len(ref_verts)
    assert np.array_equal(s["corners"], ref_verts)
    assert (s["geom_offsets"] == -1).all() and (s["field_offsets"] == -1).all()
    assert (s["geom_modes"] == 0).all() and (s["field_modes"] == 0).all()
    assert s["geom"].size == 0 and s["field"].size == 0


def test_edge_cases_read_as_the_reference_reads_them():
    with hr.Context(0) as ctx:
        ctx.load_vtu(str(VTU / "badindex.vtu"))
        c = ctx.get_scene()["corners"]
    assert np.array_equal(c[1, 2], [0, 0, 0]) and np.array_equal(c[1, 6], [0, 0, 0])
    assert len(REF["mixed_verts"]) == 4  # 12, 72, 25 and the last 12; wedge, quad, tetra skipped
    assert len(REF["nooffsets_verts"]) == 2  # the tetrahedron without offsets ends the list
    assert len(REF["badrange_verts"]) == 3
    assert len(REF["wide_verts"]) == 1


def test_no_supported_cell_fails_and_leaves_scene_unchanged(tmp_path):
    pts = " ".join("%d %d %d" % (i & 1, (i >> 1) & 1, i >> 2) for i in range(8))
    text = (f"<Points><DataArray>{pts}</DataArray></Points><Cells>"
            "<DataArray Name=\"connectivity\">0 1 2 4 1 3 2 7</DataArray>"
            "<DataArray Name=\"offsets\">4 8</DataArray>"
            "<DataArray Name=\"types\">10 10</DataArray></Cells>")
    path = broken(tmp_path, text)
    with hr.Context(0) as ctx:
        ctx.load_vtu(str(VTU / "grid.vtu"))
        before = ctx.get_scene()["corners"].copy()
        with pytest.raises(hr.HoError) as ei:
            ctx.load_vtu(path)
        assert ei.value.code == -5
        assert "no hexahedron, wedge or quad cells" in str(ei.value)
        assert np.array_equal(ctx.get_scene()["corners"], before)
        assert ctx.get_prims()["kind"].size == 0
    import oracle_bind as ob

    if ob.ref_available():
        with pytest.raises(RuntimeError):
            ob.RefScene(vtu=path)


def test_appends_to_the_scene(tmp_path):
    with hr.Context(0) as ctx:
        ctx.load_vtu(str(VTU / "grid.vtu"))
        ctx.load_vtu(str(VTU / "mixed.vtu"))
        c = ctx.get_scene()["corners"]
    assert np.array_equal(c, np.concatenate([REF["grid_verts"], REF["mixed_verts"]]))


def broken(tmp_path, text, name="x.vtu"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


@pytest.mark.parametrize("text, code", [
    ("", "io"),
    ("<VTKFile><Cells></Cells></VTKFile>", "parse"),
    ("<VTKFile><Points><DataArray format=\"ascii\">0 0 0</DataArray></Points></VTKFile>", "parse"),
    ("<Points><DataArray format=\"binary\">AAAA</DataArray></Points><Cells></Cells>", "parse"),
    ("<Points><DataArray>0 0 0 1</DataArray></Points><Cells></Cells>", "parse"),
    ("<Points><DataArray>0 0 0</DataArray></Points><Cells>"
     "<DataArray Name=\"types\">12</DataArray></Cells>", "parse"),
    ("<Points><DataArray>0 0 0</DataArray></Points><Cells>"
     "<DataArray Name=\"connectivity\">0 0 0 0 0 0 0 0</DataArray></Cells>", "parse"),
])
def test_malformed_files(tmp_path, text, code):
    path = broken(tmp_path, text) if text else broken(tmp_path, "", "empty.vtu")
    with hr.Context(0) as ctx:
        with pytest.raises(hr.HoError) as ei:
            ctx.load_vtu(path)
        assert ei.value.code == (-4 if code == "io" else -5)  # HO_ERR_IO, HO_ERR_PARSE
        assert ctx.get_scene()["corners"].shape[0] == 0
    import oracle_bind as ob

    if ob.ref_available():  # the reference loader refuses the same file
        with pytest.raises(RuntimeError):
            ob.RefScene(vtu=path)
    with hr.Context(0) as ctx:
        with pytest.raises(hr.HoError) as ei:
            ctx.load_vtu(str(tmp_path / "missing.vtu"))
        assert ei.value.code == -4


def test_minimal_file_without_offsets(tmp_path):
    pts = " ".join("%d %d %d" % (i & 1, (i >> 1) & 1, i >> 2) for i in range(8))
    text = (f"<Points><DataArray>{pts}</DataArray></Points><Cells>"
            "<DataArray Name=\"connectivity\">0 1 3 2 4 5 7 6</DataArray>"
            "<DataArray Name=\"types\">12</DataArray></Cells>")
    with hr.Context(0) as ctx:
        ctx.load_vtu(broken(tmp_path, text))
        c = ctx.get_scene()["corners"]
    assert c.shape == (1, 8, 3)
    assert np.array_equal(c[0, 2], [1, 1, 0]) and np.array_equal(c[0, 6], [1, 1, 1])
