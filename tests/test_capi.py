"""The C ABI library: it loads, exports every entry point include/horender.h
declares, and its host-only calls (scene assembly, validation, error
reporting, PPM output) behave as documented. No GPU compute here."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

import horender as hr
from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "horender.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ho_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = C.CDLL(str(hr.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_create_and_errors():
    with hr.Context(0) as ctx:
        with pytest.raises(hr.HoError) as ei:
            ctx.build_bvh()  # empty scene
        assert ei.value.code == -3 and "empty" in str(ei.value)
        with pytest.raises(hr.HoError) as ei:
            ctx.render(hr.Camera((2, 2, 2), (0, 0, 0)), [0.1], 8, 8)
        assert ei.value.code == -3
        with pytest.raises(hr.HoError) as ei:
            ctx.set_mode(17)
        assert ei.value.code == -1
    out = C.c_void_p()
    assert hr.lib.ho_create(-1, C.byref(out)) == -1


def test_generate_and_read_back():
    with hr.Context(0) as ctx:
        ctx.generate_synthetic(2, 3, 1, 2, 4, 0.05, 4, 9)
        s = ctx.get_scene()
        n = s["geom_offsets"].shape[0]
        assert n == 6
        m = s["geom_modes"][:, 0]
        assert ((m >= 3) & (m <= 5)).all()
        # offsets are consistent with modes
        sizes = 3 * np.prod(s["geom_modes"].astype(np.int64), axis=1)
        assert np.array_equal(np.cumsum(np.r_[0, sizes[:-1]]), s["geom_offsets"])
        assert s["geom"].size == sizes.sum()
        assert np.isfinite(s["geom"]).all() and np.isfinite(s["field"]).all()
        info = ctx.info()
        assert info["n_elem"] == 6 and info["n_nodes"] == 0


def test_add_hexes_validation_leaves_scene_unchanged():
    with hr.Context(0) as ctx:
        ctx.generate_synthetic(1, 1, 1, 2, 2, 0.0, 1, 1)
        s = ctx.get_scene()
        bad_modes = s["geom_modes"].copy()
        bad_modes[0, 0] = 12
        with pytest.raises(hr.HoError) as ei:
            ctx.add_hexes(s["corners"], bad_modes, s["geom"], s["geom_offsets"], s["field_modes"], s["field"],
                          s["field_offsets"])
        assert ei.value.code == -7
        with pytest.raises(hr.HoError) as ei:
            ctx.add_hexes(s["corners"], s["geom_modes"], s["geom"][:-1], s["geom_offsets"], s["field_modes"],
                          s["field"], s["field_offsets"])
        assert ei.value.code == -1
        assert ctx.info()["n_elem"] == 1
        ctx.add_hexes(s["corners"], s["geom_modes"], s["geom"], s["geom_offsets"], s["field_modes"], s["field"],
                      s["field_offsets"])
        s2 = ctx.get_scene()
        assert s2["geom_offsets"].tolist() == [0, s["geom"].size]
        assert np.array_equal(s2["geom"][: s["geom"].size], s["geom"])


@pytest.mark.parametrize("where", ["corner", "geom", "field"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_non_finite_inputs_refused(where, bad):
    """A NaN or infinite corner or coefficient is refused with HO_ERR_ARG and
    the scene is left as it was (it would otherwise reach the solvers as a NaN
    iterate); the same for a primitive's vertex."""
    with hr.Context(0) as ctx:
        ctx.generate_synthetic(1, 1, 1, 2, 2, 0.0, 1, 1)
        s = ctx.get_scene()
        arr = {"corner": s["corners"].copy(), "geom": s["geom"].copy(), "field": s["field"].copy()}
        arr[where].reshape(-1)[3] = bad
        with pytest.raises(hr.HoError) as ei:
            ctx.add_hexes(arr["corner"], s["geom_modes"], arr["geom"], s["geom_offsets"], s["field_modes"],
                          arr["field"], s["field_offsets"])
        assert ei.value.code == -1 and "non-finite" in str(ei.value)
        assert ctx.info()["n_elem"] == 1
        verts = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]]], np.float32)
        verts[0, 2, 1] = bad
        with pytest.raises(hr.HoError) as ei:
            ctx.add_quads(verts, np.zeros((1, 2), np.uint32), np.zeros(0, np.float32), np.array([-1]),
                          np.zeros((1, 2), np.uint32), np.zeros(0, np.float32), np.array([-1]))
        assert ei.value.code == -1 and ctx.info()["n_quads"] == 0


def test_trilinear_elements_accepted():
    with hr.Context(0) as ctx:
        corners = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
                           np.float32)[None]
        ctx.add_hexes(corners, np.zeros((1, 3), np.uint32), np.zeros(0, np.float32), np.array([-1]),
                      np.zeros((1, 3), np.uint32), np.zeros(0, np.float32), np.array([-1]))
        assert ctx.info()["max_modes"] == 2


def test_save_ppm(tmp_path):
    rgb = np.arange(4 * 3 * 3, dtype=np.uint8).reshape(4, 3, 3)
    p = tmp_path / "a.ppm"
    hr.save_ppm(rgb, str(p))
    data = p.read_bytes()
    assert data.startswith(b"P6\n3 4\n255\n") and data.endswith(rgb.tobytes())
    with pytest.raises(hr.HoError):
        hr.save_ppm(rgb, str(tmp_path / "no" / "such" / "dir.ppm"))


def read_png(path):
    """Chunks checked (CRC-32), IDAT inflated by zlib, filter bytes 0."""
    import struct
    import zlib

    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    at, chunks = 8, []
    while at < len(data):
        (n,) = struct.unpack(">I", data[at:at + 4])
        kind, body = data[at + 4:at + 8], data[at + 8:at + 8 + n]
        (crc,) = struct.unpack(">I", data[at + 8 + n:at + 12 + n])
        assert crc == zlib.crc32(kind + body)
        chunks.append((kind, body))
        at += 12 + n
    assert [k for k, _ in chunks] == [b"IHDR", b"IDAT", b"IEND"]
    w, h, depth, ctype, comp, filt, lace = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, lace) == (8, 2, 0, 0, 0)
    raw = np.frombuffer(zlib.decompress(chunks[1][1]), np.uint8).reshape(h, 1 + 3 * w)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, 3)


@pytest.mark.parametrize("shape", [(4, 3), (1, 1), (200, 151)])
def test_save_png(tmp_path, shape):
    """The PNG holds the same pixels as the PPM, in the same row order; the
    200 x 151 image spans two stored deflate blocks."""
    h, w = shape
    rgb = np.random.default_rng(h * w).integers(0, 256, (h, w, 3), dtype=np.uint8)
    p = tmp_path / "a.png"
    hr.save_png(rgb, str(p))
    assert np.array_equal(read_png(p), rgb)
    with pytest.raises(hr.HoError):
        hr.save_png(rgb, str(tmp_path / "no" / "such" / "dir.png"))


def test_engine_options():
    with hr.Context(0) as ctx:
        assert ctx.get_option(hr.OPT_GRAPH) == 1
        assert ctx.get_option(hr.OPT_ROUNDS) == 16
        assert ctx.get_option(hr.OPT_ROUND_CHUNK) == 20
        ctx.set_option(hr.OPT_TENSOR, 1)
        assert ctx.get_option(hr.OPT_ROUND_CHUNK) == 80  # 4 warps x 20 slots (tensor-core form)
        ctx.set_option(hr.OPT_TENSOR, 0)
        assert ctx.get_option(hr.OPT_FP64_CHECK) == 1
        assert ctx.get_option(hr.OPT_TIME_ROUNDS) == 0
        assert ctx.get_option(hr.OPT_TENSOR) == 0
        assert ctx.get_option(hr.OPT_TAIL) == 4
        assert ctx.get_option(hr.OPT_GPU_FIT) == -1 and ctx.get_option(hr.OPT_LAST_FIT_GPU) == 0
        ctx.set_option(hr.OPT_TIME_ROUNDS, 1)
        assert ctx.get_option(hr.OPT_TIME_ROUNDS) == 1
        ctx.set_option(hr.OPT_GRAPH, 0)
        ctx.set_option(hr.OPT_ROUNDS, 3)
        ctx.set_option(hr.OPT_ROUND_CHUNK, 200)
        assert (ctx.get_option(hr.OPT_GRAPH), ctx.get_option(hr.OPT_ROUNDS), ctx.get_option(hr.OPT_ROUND_CHUNK)) == (
            0, 3, 200)
        for opt, bad in ((hr.OPT_GRAPH, 2), (hr.OPT_ROUNDS, 0), (hr.OPT_ROUNDS, 257), (hr.OPT_ROUND_CHUNK, 0),
                         (hr.OPT_ROUND_CHUNK, 4097), (hr.OPT_TIME_ROUNDS, 2), (hr.OPT_TENSOR, -1),
                         (hr.OPT_TAIL, -1), (hr.OPT_TAIL, 257), (hr.OPT_GPU_FIT, 2)):
            with pytest.raises(hr.HoError) as ei:
                ctx.set_option(opt, bad)
            assert ei.value.code == -7
        with pytest.raises(hr.HoError) as ei:
            ctx.set_option(99, 1)
        assert ei.value.code == -1
        assert ctx.get_option(hr.OPT_ROUNDS) == 3  # a refused value leaves the option unchanged
