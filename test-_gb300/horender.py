"""Python binding of libhorender.so (the C ABI in include/horender.h).

This is the interface tests and benchmarks drive; it adds no computation of
its own. It mirrors the reference's host API shape: load a scene (or add
hexes / generate a seeded one), build the BVH, render(camera, isovalues) ->
images, intersect(rays) -> hits, save_ppm.

There is no fallback: if the compiled library is missing, importing this
module raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from workloads import (ISO_POOL, MULTIVIEW, PATHS, RESOLUTIONS, WORKLOADS, Camera, Workload,  # noqa: F401
                       sphere_views)

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libhorender.so"

HO_OK = 0
ERRORS = {-1: "HO_ERR_ARG", -2: "HO_ERR_CUDA", -3: "HO_ERR_STATE", -4: "HO_ERR_IO", -5: "HO_ERR_PARSE",
          -6: "HO_ERR_NOMEM", -7: "HO_ERR_RANGE", -8: "HO_ERR_DEVICE"}
MODE_PLAIN, MODE_LEARNED, MODE_BATCHED = 0, 1, 2
OPT_GRAPH, OPT_ROUNDS, OPT_ROUND_CHUNK, OPT_FP64_CHECK, OPT_TIME_ROUNDS, OPT_TENSOR, OPT_TAIL = 1, 2, 3, 4, 5, 6, 7
OPT_GPU_FIT, OPT_LAST_FIT_GPU, OPT_WARM_CAP = 8, 9, 10
MLP_PARAMS, MLP_IN, MLP_OUT = 40328, 48, 8
NOALLOC_MAX_RAYS = 32768
HIT_MISS, HIT_FACE, HIT_ISO = 0, 1, 2
HIT_PRISM, HIT_QUAD, HIT_TRI = 3, 4, 5
FLAG_FALLBACK, FLAG_FP64_FAIL, FLAG_OVERFLOW, FLAG_INCOMPLETE, FLAG_TIE, FLAG_GRAZING = 1, 2, 4, 8, 16, 32

HIT_DTYPE = np.dtype([("t", "<f4"), ("elem", "<i4"), ("face", "<i2"), ("kind", "<i2"), ("xi", "<f4", 3),
                      ("n", "<f4", 3), ("u", "<f4"), ("flags", "<u4"), ("iters", "<u4")])
assert HIT_DTYPE.itemsize == 48


class HoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class _Camera(C.Structure):
    _fields_ = [("lookfrom", C.c_float * 3), ("lookat", C.c_float * 3), ("vup", C.c_float * 3),
                ("vfov_deg", C.c_float), ("focus_dist", C.c_float)]


class _Synth(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("order_min", C.c_int32),
                ("order_max", C.c_int32), ("curve_amp", C.c_double), ("n_gauss", C.c_int32),
                ("seed", C.c_uint64)]


class _Info(C.Structure):
    _fields_ = [("n_elem", C.c_int64), ("n_nodes", C.c_int64), ("max_modes", C.c_int32),
                ("bvh_depth", C.c_int32), ("device_bytes", C.c_int64), ("bounds", C.c_float * 6),
                ("n_prisms", C.c_int64), ("n_quads", C.c_int64), ("n_tris", C.c_int64)]


class _Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("rays", "candidates", "geom_evals", "map_evals", "field_evals",
                                          "newton_iters", "face_iters", "faces_culled", "node_visits",
                                          "mlp_accepted", "mlp_rejected", "restarts")] + [
        ("max_modes", C.c_int32), ("status", C.c_int32), ("phase_cycles", C.c_uint64 * 4),
        ("rounds", C.c_uint64), ("round_pairs", C.c_uint64), ("solve_steps", C.c_uint64),
        ("lane_steps", C.c_uint64), ("graph", C.c_uint64), ("fp64_checked", C.c_uint64),
        ("fp64_failed", C.c_uint64), ("fp64_failed_after_fallback", C.c_uint64), ("round_flops", C.c_uint64),
        ("kernel_launches", C.c_uint64), ("round_kernel_ns", C.c_uint64), ("round_launches", C.c_uint64),
        ("tail_rays", C.c_uint64), ("prim_candidates", C.c_uint64), ("prim_iters", C.c_uint64),
        ("prim_flops", C.c_uint64), ("prim_kernel_ns", C.c_uint64), ("prim_node_visits", C.c_uint64),
        ("fp64_polished", C.c_uint64), ("fp64_ties", C.c_uint64), ("fp64_ties_swapped", C.c_uint64),
        ("grazing_hits", C.c_uint64)]


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() (no CPU fallback exists)")
    L = C.CDLL(str(LIB_PATH))
    vp, i32, i64, f32 = C.c_void_p, C.c_int, C.c_int64, C.c_float
    L.ho_create.argtypes = [i32, C.POINTER(vp)]
    L.ho_destroy.argtypes = [vp]
    L.ho_destroy.restype = None
    L.ho_last_error.argtypes = [vp]
    L.ho_last_error.restype = C.c_char_p
    L.ho_load_xml_fld.argtypes = [vp, C.c_char_p, C.c_char_p]
    L.ho_load_vtu.argtypes = [vp, C.c_char_p]
    L.ho_add_hexes.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, vp, i64, vp]
    for f in (L.ho_add_prisms, L.ho_add_quads, L.ho_add_tris):
        f.argtypes = [vp, i64, vp, vp, vp, i64, vp, vp, vp, i64, vp]
    L.ho_get_prims.argtypes = [vp] + [vp] * 11
    L.ho_get_prim_boxes.argtypes = [vp, vp]
    L.ho_generate_synthetic.argtypes = [vp, C.POINTER(_Synth)]
    L.ho_get_scene.argtypes = [vp] + [vp] * 10
    L.ho_build_bvh.argtypes = [vp]
    L.ho_scene_info_get.argtypes = [vp, C.POINTER(_Info)]
    L.ho_get_boxes.argtypes = [vp, vp]
    L.ho_get_hull_boxes.argtypes = [vp, vp, vp]
    L.ho_render.argtypes = [vp, C.POINTER(_Camera), vp, i32, i32, i32, i32, vp, vp]
    L.ho_render_views.argtypes = [vp, i32, vp, vp, vp, vp, vp, i32, vp, vp, vp]
    L.ho_render_views_device.argtypes = [vp, i32, vp, vp, vp, vp, vp, i32, vp, vp, vp, vp]
    L.ho_render_device.argtypes = [vp, C.POINTER(_Camera), vp, i32, i32, i32, i32, vp, vp, vp]
    L.ho_render_tile.argtypes = [vp, C.POINTER(_Camera), vp, i32, i32, i32, i32, i32, i32, i32, i32, vp, vp]
    L.ho_render_tile_device.argtypes = [vp, C.POINTER(_Camera), vp, i32, i32, i32, i32, i32, i32, i32, i32, vp, vp,
                                        vp]
    L.ho_path_trace.argtypes = [vp, C.POINTER(_Camera), vp, i32, i32, i32, i32, i32, C.c_uint64, i32, vp,
                                C.POINTER(i64)]
    L.ho_path_trace_device.argtypes = [vp, C.POINTER(_Camera), vp, i32, i32, i32, i32, i32, C.c_uint64, i32, vp,
                                       C.POINTER(i64), vp]
    L.ho_intersect.argtypes = [vp, i64, vp, f32, i32, vp]
    L.ho_hit_residuals.argtypes = [vp, i64, vp, vp, vp]
    L.ho_intersect_device.argtypes = [vp, i64, vp, f32, i32, vp, vp]
    L.ho_intersect_soa.argtypes = [vp, i64, vp, f32, i32, vp]
    L.ho_set_mode.argtypes = [vp, i32]
    L.ho_set_option.argtypes = [vp, i32, i64]
    L.ho_get_option.argtypes = [vp, i32, C.POINTER(C.c_int64)]
    L.ho_autotune.argtypes = [vp, C.POINTER(_Camera), vp, i32, i32, i32, i32, C.POINTER(C.c_int64), vp, vp]
    L.ho_get_stats.argtypes = [vp, C.POINTER(_Stats)]
    L.ho_save_ppm.argtypes = [vp, i32, i32, C.c_char_p]
    L.ho_save_png.argtypes = [vp, i32, i32, C.c_char_p]
    L.ho_measure_fp32_peak.argtypes = [i32, C.POINTER(C.c_double)]
    L.ho_intersect_device_noalloc.argtypes = [vp, i64, vp, f32, i32, vp, vp]
    L.ho_mlp_init.argtypes = [vp, C.c_uint64]
    L.ho_mlp_set_params.argtypes = [vp, vp]
    L.ho_mlp_get_params.argtypes = [vp, vp]
    L.ho_mlp_forward.argtypes = [vp, vp, i64, vp]
    L.ho_mlp_grad.argtypes = [vp, vp, vp, vp, i32, vp, vp]
    L.ho_learn_samples.argtypes = [vp, i64, C.c_uint64, vp, vp, vp]
    L.ho_train_mlp.argtypes = [vp, i64, i32, i32, f32, C.c_uint64, vp]
    L.ho_mlp_save.argtypes = [vp, C.c_char_p]
    L.ho_mlp_load.argtypes = [vp, C.c_char_p]
    return L


lib = _load()


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def _cam(cam: Camera) -> _Camera:
    c = _Camera()
    c.lookfrom[:] = [float(x) for x in cam.lookfrom]
    c.lookat[:] = [float(x) for x in cam.lookat]
    c.vup[:] = [float(x) for x in cam.vup]
    c.vfov_deg = float(cam.vfov_deg)
    c.focus_dist = float(cam.focus_dist)
    return c




class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib.ho_create(int(device), C.byref(h))
        if rc != HO_OK:
            raise HoError(rc, "ho_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib.ho_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc: int):
        if rc != HO_OK:
            raise HoError(rc, lib.ho_last_error(self.h).decode())

    # ---- scene ---------------------------------------------------------------
    def add_hexes(self, corners, geom_modes, geom, geom_offsets, field_modes, field, field_offsets):
        corners = np.ascontiguousarray(corners, np.float32)
        gm = np.ascontiguousarray(geom_modes, np.uint32)
        geom = np.ascontiguousarray(geom, np.float32)
        go = np.ascontiguousarray(geom_offsets, np.int64)
        fm = np.ascontiguousarray(field_modes, np.uint32)
        field = np.ascontiguousarray(field, np.float32)
        fo = np.ascontiguousarray(field_offsets, np.int64)
        n = go.shape[0]
        self._ck(lib.ho_add_hexes(self.h, n, _p(corners), _p(gm), _p(geom), geom.size, _p(go), _p(fm), _p(field),
                                  field.size, _p(fo)))

    def _add_prims(self, fn, dims, verts, geom_modes, geom, geom_offsets, field_modes, field, field_offsets):
        verts = np.ascontiguousarray(verts, np.float32)
        go = np.ascontiguousarray(geom_offsets, np.int64).reshape(-1)
        n = go.shape[0]
        gm = np.ascontiguousarray(geom_modes, np.uint32).reshape(n, dims)
        fm = np.ascontiguousarray(field_modes, np.uint32).reshape(n, dims)
        geom = np.ascontiguousarray(geom, np.float32)
        field = np.ascontiguousarray(field, np.float32)
        fo = np.ascontiguousarray(field_offsets, np.int64).reshape(-1)
        self._ck(fn(self.h, n, _p(verts), _p(gm), _p(geom), geom.size, _p(go), _p(fm), _p(field), field.size, _p(fo)))

    def add_prisms(self, verts, geom_modes, geom, geom_offsets, field_modes, field, field_offsets):
        """verts n x 6 x 3; modes n x 3 (see ho_add_prisms)."""
        self._add_prims(lib.ho_add_prisms, 3, verts, geom_modes, geom, geom_offsets, field_modes, field, field_offsets)

    def add_quads(self, verts, geom_modes, geom, geom_offsets, field_modes, field, field_offsets):
        """verts n x 4 x 3; modes n x 2."""
        self._add_prims(lib.ho_add_quads, 2, verts, geom_modes, geom, geom_offsets, field_modes, field, field_offsets)

    def add_tris(self, verts, geom_modes, geom, geom_offsets, field_modes, field, field_offsets):
        """verts n x 3 x 3; modes n x 2."""
        self._add_prims(lib.ho_add_tris, 2, verts, geom_modes, geom, geom_offsets, field_modes, field, field_offsets)

    def add_prim_arrays(self, arrs):
        """Add every primitive of a kind-major list (kind, verts n x 6 x 3, modes
        n x 3, offsets into one geometry and one field pool)."""
        fns = {0: (self.add_prisms, 6, 3), 1: (self.add_quads, 4, 2), 2: (self.add_tris, 3, 2)}
        for k, (fn, nv, dims) in fns.items():
            m = np.asarray(arrs.kind) == k
            if m.any():
                fn(np.asarray(arrs.verts)[m][:, :nv], np.asarray(arrs.geom_modes)[m][:, :dims], arrs.geom,
                   np.asarray(arrs.geom_offset)[m], np.asarray(arrs.field_modes)[m][:, :dims], arrs.field,
                   np.asarray(arrs.field_offset)[m])

    def get_prims(self) -> dict:
        """The scene's prisms, quads and triangles, kind-major (ho_get_prims)."""
        n, gl, fl = C.c_int64(), C.c_int64(), C.c_int64()
        self._ck(lib.ho_get_prims(self.h, C.byref(n), None, None, None, None, C.byref(gl), None, None, None,
                                  C.byref(fl), None))
        n = n.value
        out = dict(kind=np.zeros(n, np.int32), verts=np.zeros((n, 6, 3), np.float32),
                   geom_modes=np.zeros((n, 3), np.uint32), geom=np.zeros(gl.value, np.float32),
                   geom_offsets=np.zeros(n, np.int64), field_modes=np.zeros((n, 3), np.uint32),
                   field=np.zeros(fl.value, np.float32), field_offsets=np.zeros(n, np.int64))
        self._ck(lib.ho_get_prims(self.h, None, _p(out["kind"]), _p(out["verts"]), _p(out["geom_modes"]),
                                  _p(out["geom"]), None, _p(out["geom_offsets"]), _p(out["field_modes"]),
                                  _p(out["field"]), None, _p(out["field_offsets"])))
        return out

    def prim_boxes(self) -> np.ndarray:
        i = self.info()
        out = np.zeros((i["n_prisms"] + i["n_quads"] + i["n_tris"], 6), np.float32)
        self._ck(lib.ho_get_prim_boxes(self.h, _p(out)))
        return out

    def generate_synthetic(self, nx, ny, nz, order_min, order_max, curve_amp, n_gauss, seed):
        s = _Synth(nx, ny, nz, order_min, order_max, curve_amp, n_gauss, seed)
        self._ck(lib.ho_generate_synthetic(self.h, C.byref(s)))

    def load_xml_fld(self, xml: str, fld: str):
        self._ck(lib.ho_load_xml_fld(self.h, str(xml).encode(), str(fld).encode()))

    def load_vtu(self, path: str):
        self._ck(lib.ho_load_vtu(self.h, str(path).encode()))

    def get_scene(self) -> dict:
        n, gl, fl = C.c_int64(), C.c_int64(), C.c_int64()
        self._ck(lib.ho_get_scene(self.h, C.byref(n), None, None, None, C.byref(gl), None, None, None, C.byref(fl),
                                  None))
        n = n.value
        out = dict(corners=np.zeros((n, 8, 3), np.float32), geom_modes=np.zeros((n, 3), np.uint32),
                   geom=np.zeros(gl.value, np.float32), geom_offsets=np.zeros(n, np.int64),
                   field_modes=np.zeros((n, 3), np.uint32), field=np.zeros(fl.value, np.float32),
                   field_offsets=np.zeros(n, np.int64))
        self._ck(lib.ho_get_scene(self.h, None, _p(out["corners"]), _p(out["geom_modes"]), _p(out["geom"]), None,
                                  _p(out["geom_offsets"]), _p(out["field_modes"]), _p(out["field"]), None,
                                  _p(out["field_offsets"])))
        return out

    def build_bvh(self):
        self._ck(lib.ho_build_bvh(self.h))

    def info(self) -> dict:
        i = _Info()
        self._ck(lib.ho_scene_info_get(self.h, C.byref(i)))
        return dict(n_elem=i.n_elem, n_nodes=i.n_nodes, max_modes=i.max_modes, bvh_depth=i.bvh_depth,
                    device_bytes=i.device_bytes, bounds=list(i.bounds), n_prisms=i.n_prisms, n_quads=i.n_quads,
                    n_tris=i.n_tris)

    def boxes(self) -> np.ndarray:
        n = self.info()["n_elem"]
        out = np.zeros((n, 6), np.float32)
        self._ck(lib.ho_get_boxes(self.h, _p(out)))
        return out

    def hull_boxes(self):
        n = self.info()["n_elem"]
        hull = np.zeros((n, 6), np.float32)
        faces = np.zeros((n, 6, 6), np.float32)
        self._ck(lib.ho_get_hull_boxes(self.h, _p(hull), _p(faces)))
        return hull, faces

    def set_mode(self, mode: int):
        self._ck(lib.ho_set_mode(self.h, int(mode)))

    def set_option(self, option: int, value: int):
        self._ck(lib.ho_set_option(self.h, int(option), int(value)))

    def autotune(self, cam: "Camera", isovalues, width: int, height: int, iso_zero_disables: bool = False) -> dict:
        """Pick the element batch size of the round kernel for this render
        (ho_autotune); returns the chosen size and every candidate's time."""
        iso = np.ascontiguousarray(isovalues, dtype=np.float32)
        chunk = C.c_int64()
        cand = np.zeros(5, np.int64)
        ms = np.zeros(5, np.float32)
        self._ck(lib.ho_autotune(self.h, C.byref(_cam(cam)), _p(iso), iso.size, int(width), int(height),
                                 int(bool(iso_zero_disables)), C.byref(chunk), _p(cand), _p(ms)))
        return {"chunk": chunk.value, "candidates": cand.tolist(), "ms": ms.tolist()}

    def get_option(self, option: int) -> int:
        v = C.c_int64()
        self._ck(lib.ho_get_option(self.h, int(option), C.byref(v)))
        return v.value

    # ---- queries ---------------------------------------------------------------
    def render(self, camera: Camera, isovalues, width: int, height: int, iso_zero_disables: bool = True,
               want_rgb: bool = True, want_hits: bool = False, rgb_out: np.ndarray | None = None):
        iso = np.ascontiguousarray(isovalues, np.float32).reshape(-1)
        n = iso.size
        if rgb_out is not None:
            assert rgb_out.dtype == np.uint8 and rgb_out.size == n * height * width * 3 and rgb_out.flags.c_contiguous
            rgb = rgb_out
        else:
            rgb = np.zeros((n, height, width, 3), np.uint8) if want_rgb else None
        hits = np.zeros((n, height, width), HIT_DTYPE) if want_hits else None
        cam = _cam(camera)
        self._ck(lib.ho_render(self.h, C.byref(cam), _p(iso), n, width, height, int(iso_zero_disables),
                               _p(rgb) if rgb is not None else None, _p(hits) if hits is not None else None))
        return rgb, hits

    @staticmethod
    def _views(cameras, widths, heights, isovalues):
        n = len(cameras)
        cams = (_Camera * n)(*[_cam(c) for c in cameras])
        w = np.ascontiguousarray(widths, np.int32)
        h = np.ascontiguousarray(heights, np.int32)
        iso = np.zeros((n, 8), np.float32)
        n_iso = np.zeros(n, np.int32)
        for v, vals in enumerate(isovalues):
            vals = np.atleast_1d(np.asarray(vals, np.float32))
            iso[v, :vals.size] = vals
            n_iso[v] = vals.size
        total = int((w.astype(np.int64) * h * n_iso).sum())
        return n, cams, w, h, iso, n_iso, total

    def render_views(self, cameras, widths, heights, isovalues, iso_zero_disables: bool = False,
                     want_rgb: bool = True, want_hits: bool = False, rgb_out: np.ndarray | None = None):
        """Many views in one call (ho_render_views). isovalues[v] lists view
        v's isovalues. Returns flat rgb (total x 3) and hits (total), and the
        query offset of each view (n + 1 entries)."""
        n, cams, w, h, iso, n_iso, total = self._views(cameras, widths, heights, isovalues)
        if rgb_out is not None:
            assert rgb_out.dtype == np.uint8 and rgb_out.size == total * 3 and rgb_out.flags.c_contiguous
            rgb = rgb_out
        else:
            rgb = np.zeros((total, 3), np.uint8) if want_rgb else None
        hits = np.zeros(total, HIT_DTYPE) if want_hits else None
        offs = np.zeros(n + 1, np.int64)
        self._ck(lib.ho_render_views(self.h, n, C.cast(cams, C.c_void_p), _p(w), _p(h), _p(iso), _p(n_iso),
                                     int(iso_zero_disables), _p(rgb) if rgb is not None else None,
                                     _p(hits) if hits is not None else None, _p(offs)))
        return rgb, hits, offs

    def render_views_device(self, cameras, widths, heights, isovalues, rgb_ptr, hits_ptr, stream_ptr,
                            iso_zero_disables: bool = False) -> np.ndarray:
        n, cams, w, h, iso, n_iso, total = self._views(cameras, widths, heights, isovalues)
        offs = np.zeros(n + 1, np.int64)
        self._ck(lib.ho_render_views_device(self.h, n, C.cast(cams, C.c_void_p), _p(w), _p(h), _p(iso), _p(n_iso),
                                            int(iso_zero_disables), rgb_ptr, hits_ptr, _p(offs), stream_ptr))
        return offs

    def render_tile(self, camera: Camera, isovalues, width: int, height: int, x0: int, y0: int, tile_w: int,
                    tile_h: int, iso_zero_disables: bool = True, want_rgb: bool = True, want_hits: bool = False,
                    rgb_out: np.ndarray | None = None):
        """The tile_w x tile_h pixels at (x0, y0) of the width x height render:
        images (n_iso, tile_h, tile_w, 3) and hits, equal to that part of render()."""
        iso = np.ascontiguousarray(isovalues, np.float32).reshape(-1)
        n = iso.size
        if rgb_out is not None:
            assert rgb_out.dtype == np.uint8 and rgb_out.size == n * tile_h * tile_w * 3 and rgb_out.flags.c_contiguous
            rgb = rgb_out
        else:
            rgb = np.zeros((n, tile_h, tile_w, 3), np.uint8) if want_rgb else None
        hits = np.zeros((n, tile_h, tile_w), HIT_DTYPE) if want_hits else None
        cam = _cam(camera)
        self._ck(lib.ho_render_tile(self.h, C.byref(cam), _p(iso), n, width, height, x0, y0, tile_w, tile_h,
                                    int(iso_zero_disables), _p(rgb) if rgb is not None else None,
                                    _p(hits) if hits is not None else None))
        return rgb, hits

    def render_tile_device(self, camera: Camera, isovalues, width, height, x0, y0, tile_w, tile_h, rgb_ptr, hits_ptr,
                           stream_ptr, iso_zero_disables: bool = True):
        iso = np.ascontiguousarray(isovalues, np.float32).reshape(-1)
        cam = _cam(camera)
        self._ck(lib.ho_render_tile_device(self.h, C.byref(cam), _p(iso), iso.size, width, height, x0, y0, tile_w,
                                           tile_h, int(iso_zero_disables), rgb_ptr, hits_ptr, stream_ptr))

    def render_device(self, camera: Camera, isovalues, width, height, rgb_ptr, hits_ptr, stream_ptr,
                      iso_zero_disables: bool = True):
        iso = np.ascontiguousarray(isovalues, np.float32).reshape(-1)
        cam = _cam(camera)
        self._ck(lib.ho_render_device(self.h, C.byref(cam), _p(iso), iso.size, width, height,
                                      int(iso_zero_disables), rgb_ptr, hits_ptr, stream_ptr))

    def path_trace(self, camera: Camera, isovalues, width, height, spp=1, max_depth=4, seed=1,
                   iso_zero_disables: bool = True):
        """Path-traced images (n_iso, H, W, 3) uint8 and the ray queries traced."""
        iso = np.ascontiguousarray(isovalues, np.float32).reshape(-1)
        out = np.zeros((iso.size, height, width, 3), np.uint8)
        rays = C.c_int64(0)
        cam = _cam(camera)
        self._ck(lib.ho_path_trace(self.h, C.byref(cam), _p(iso), iso.size, width, height, int(spp), int(max_depth),
                                   int(seed), int(iso_zero_disables), _p(out), C.byref(rays)))
        return out, int(rays.value)

    def path_trace_device(self, camera: Camera, isovalues, width, height, rgb_ptr, stream_ptr, spp=1, max_depth=4,
                          seed=1, iso_zero_disables: bool = True) -> int:
        iso = np.ascontiguousarray(isovalues, np.float32).reshape(-1)
        rays = C.c_int64(0)
        cam = _cam(camera)
        self._ck(lib.ho_path_trace_device(self.h, C.byref(cam), _p(iso), iso.size, width, height, int(spp),
                                          int(max_depth), int(seed), int(iso_zero_disables), rgb_ptr, C.byref(rays),
                                          stream_ptr))
        return int(rays.value)

    def intersect(self, rays: np.ndarray, iso: float, iso_enabled: bool = True) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.zeros(rays.shape[0], HIT_DTYPE)
        self._ck(lib.ho_intersect(self.h, rays.shape[0], _p(rays), float(iso), int(iso_enabled), _p(out)))
        return out

    def intersect_soa(self, ray_soa: np.ndarray, iso: float, iso_enabled: bool = True) -> np.ndarray:
        """ho_intersect_soa: ray_soa is (6, n) (origin x, y, z, direction x, y, z)."""
        ray_soa = np.ascontiguousarray(ray_soa, np.float32).reshape(6, -1)
        out = np.zeros(ray_soa.shape[1], HIT_DTYPE)
        self._ck(lib.ho_intersect_soa(self.h, ray_soa.shape[1], _p(ray_soa), float(iso), int(iso_enabled), _p(out)))
        return out

    def hit_residuals(self, rays: np.ndarray, hits: np.ndarray) -> np.ndarray:
        """The final FP64 check's residuals for the given hits: (n, 2) with
        the largest position-residual component and the field value at xi."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        hits = np.ascontiguousarray(hits, HIT_DTYPE).reshape(-1)
        out = np.zeros((rays.shape[0], 2), np.float64)
        self._ck(lib.ho_hit_residuals(self.h, rays.shape[0], _p(rays), _p(hits), _p(out)))
        return out

    def intersect_device(self, n: int, rays_ptr: int, iso: float, iso_enabled: bool, out_ptr: int, stream_ptr):
        self._ck(lib.ho_intersect_device(self.h, int(n), rays_ptr, float(iso), int(iso_enabled), out_ptr,
                                         stream_ptr))

    # ---- learned mode ----------------------------------------------------------
    def mlp_init(self, seed: int = 0):
        self._ck(lib.ho_mlp_init(self.h, int(seed)))

    def mlp_params(self) -> np.ndarray:
        out = np.zeros(MLP_PARAMS, np.float32)
        self._ck(lib.ho_mlp_get_params(self.h, _p(out)))
        return out

    def mlp_set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == MLP_PARAMS
        self._ck(lib.ho_mlp_set_params(self.h, _p(p)))

    def mlp_forward(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32).reshape(-1, MLP_IN)
        Y = np.zeros((X.shape[0], MLP_OUT), np.float32)
        self._ck(lib.ho_mlp_forward(self.h, _p(X), X.shape[0], _p(Y)))
        return Y

    def mlp_grad(self, X, T, valid):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, MLP_IN)
        T = np.ascontiguousarray(T, np.float32).reshape(-1, MLP_OUT)
        valid = np.ascontiguousarray(valid, np.uint8)
        loss = np.zeros(1, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        self._ck(lib.ho_mlp_grad(self.h, _p(X), _p(T), _p(valid), X.shape[0], _p(loss), _p(g)))
        return float(loss[0]), g

    def learn_samples(self, n: int, seed: int = 0):
        X = np.zeros((n, MLP_IN), np.float32)
        T = np.zeros((n, MLP_OUT), np.float32)
        V = np.zeros(n, np.uint8)
        self._ck(lib.ho_learn_samples(self.h, n, int(seed), _p(X), _p(T), _p(V)))
        return X, T, V

    def train_mlp(self, n_samples=2_000_000, steps=1500, batch=4096, lr=2e-3, seed=0) -> np.ndarray:
        losses = np.zeros(steps, np.float32)
        self._ck(lib.ho_train_mlp(self.h, int(n_samples), int(steps), int(batch), float(lr), int(seed), _p(losses)))
        return losses

    def mlp_save(self, path: str):
        self._ck(lib.ho_mlp_save(self.h, str(path).encode()))

    def mlp_load(self, path: str):
        self._ck(lib.ho_mlp_load(self.h, str(path).encode()))

    def intersect_device_noalloc(self, n: int, rays_ptr: int, iso: float, iso_enabled: bool, out_ptr: int,
                                 stream_ptr):
        """Batched-mode ray queries that never call the CUDA allocator (scratch
        in a fixed device array; at most NOALLOC_MAX_RAYS rays per call)."""
        self._ck(lib.ho_intersect_device_noalloc(self.h, int(n), rays_ptr, float(iso), int(iso_enabled), out_ptr,
                                                 stream_ptr))

    def stats(self) -> dict:
        s = _Stats()
        self._ck(lib.ho_get_stats(self.h, C.byref(s)))
        d = {k: getattr(s, k) for k, _ in _Stats._fields_}
        d["phase_cycles"] = dict(zip(("traversal", "iso_scan", "refine", "faces"), list(s.phase_cycles)))
        return d


def fp32_fma_peak_tflops(device: int = 0) -> float:
    v = C.c_double()
    rc = lib.ho_measure_fp32_peak(int(device), C.byref(v))
    if rc != HO_OK:
        raise HoError(rc, "FP32 peak probe failed")
    return v.value


def save_ppm(rgb: np.ndarray, path: str):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    h, w = rgb.shape[:2]
    rc = lib.ho_save_ppm(_p(rgb), w, h, str(path).encode())
    if rc != HO_OK:
        raise HoError(rc, f"cannot write {path}")


def save_png(rgb: np.ndarray, path: str):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    h, w = rgb.shape[:2]
    rc = lib.ho_save_png(_p(rgb), w, h, str(path).encode())
    if rc != HO_OK:
        raise HoError(rc, f"cannot write {path}")


def workload_context(name: str, device: int = 0, build: bool = True) -> tuple[Context, Workload]:
    w = WORKLOADS[name]
    ctx = Context(device)
    ctx.generate_synthetic(**w.synth())
    if build:
        ctx.build_bvh()
    return ctx, w
