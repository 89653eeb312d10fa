"""ctypes bindings for the CPU oracle (oracle/_build/libhorender_oracle.so)
and, where it was built, for the reference shim (oracle/_ref/libref.so).

Test infrastructure: only tests, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline arm use this module, always as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_SO = ROOT / "oracle" / "_build" / "libhorender_oracle.so"
REF_SO = ROOT / "oracle" / "_ref" / "libref.so"

HIT_DTYPE = np.dtype(
    [("t", "f8"), ("elem", "i4"), ("face", "i4"), ("kind", "i4"), ("pad", "i4"),
     ("xi", "f8", 3), ("n", "f8", 3), ("u", "f8")]
)

KIND_MISS, KIND_FACE, KIND_ISO = 0, 1, 2


class _SceneDesc(C.Structure):
    _fields_ = [
        ("n_elem", C.c_int32),
        ("geom_modes", C.c_void_p),
        ("geom_offset", C.c_void_p),
        ("geom", C.c_void_p),
        ("field_modes", C.c_void_p),
        ("field_offset", C.c_void_p),
        ("field", C.c_void_p),
        ("verts", C.c_void_p),
    ]


class _PrimsDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("kind", C.c_void_p),
        ("verts", C.c_void_p),
        ("geom_modes", C.c_void_p),
        ("geom_offset", C.c_void_p),
        ("geom", C.c_void_p),
        ("geom_len", C.c_int64),
        ("field_modes", C.c_void_p),
        ("field_offset", C.c_void_p),
        ("field", C.c_void_p),
        ("field_len", C.c_int64),
    ]


class _SynthParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("order_min", C.c_int32),
                ("order_max", C.c_int32), ("curve_amp", C.c_double), ("n_gauss", C.c_int32), ("seed", C.c_uint64)]


class _Counters(C.Structure):
    _fields_ = [("newton_iters", C.c_uint64), ("face_iters", C.c_uint64),
                ("newton_solves", C.c_uint64), ("candidates", C.c_uint64)]


def build_oracle() -> Path:
    """Compile the oracle with its Makefile (quick; no GPU needed)."""
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    return ORACLE_SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not ORACLE_SO.exists():
            build_oracle()
        L = C.CDLL(str(ORACLE_SO))
        vp, i32, i64, f32 = C.c_void_p, C.c_int, C.c_int64, C.c_float
        L.hor_scene_create.restype = vp
        L.hor_scene_create.argtypes = [C.POINTER(_SceneDesc)]
        L.hor_scene_destroy.argtypes = [vp]
        L.hor_scene_boxes.argtypes = [vp, i32, vp]
        L.hor_trace.argtypes = [vp, i32, vp, i64, f32, i32, i32, vp, C.POINTER(_Counters)]
        L.hor_map_point.argtypes = [vp, i32, i32, vp, i64, vp]
        L.hor_eval_point.argtypes = [vp, i32, i32, vp, i64, vp]
        L.hor_inverse_map.argtypes = [vp, i32, i32, vp, i64, vp]
        L.hor_find_iso.argtypes = [vp, i32, i32, vp, vp, i64, f32, vp]
        L.hor_hit_hex.argtypes = [vp, i32, i32, vp, vp, i64, vp]
        L.hor_basis.argtypes = [i32, C.c_uint, C.c_double, vp]
        L.hor_camera_rays.argtypes = [vp, vp, vp, f32, i32, i32, vp]
        L.hor_shade.argtypes = [vp, vp, i64, vp]
        L.hor_trace_replay.argtypes = [vp, i32, vp, i64, f32, i32, vp, i32, vp, vp]
        L.hor_prims_create.restype = vp
        L.hor_prims_create.argtypes = [C.POINTER(_PrimsDesc)]
        L.hor_prims_destroy.argtypes = [vp]
        L.hor_prims_boxes.argtypes = [vp, i32, vp]
        L.hor_prims_intersect.argtypes = [vp, i32, i32, vp, i64, vp, vp]
        L.hor_prims_map.argtypes = [vp, i32, i32, vp, i64, vp]
        L.hor_prims_trace.argtypes = [vp, i32, vp, i64, vp, i32]
        L.hor_synth_sizes.argtypes = [C.POINTER(_SynthParams), vp, vp, vp]
        L.hor_synth_fill.argtypes = [C.POINTER(_SynthParams), i32, vp, vp, vp, vp, vp, vp, vp]
        L.hor_polish.argtypes = [vp, vp, i64, f32, vp, i32]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class SceneArrays:
    """Flat scene arrays shared by the oracle, the reference shim and the
    product's C-ABI: per element geometry/field modes (n x 3 uint32), offsets
    (int64, -1 = absent) into flat fp32 coefficient arrays, corner vertices
    (n x 8 x 3 fp32, XML order)."""

    def __init__(self, geom_modes, geom_offset, geom, field_modes, field_offset, field, verts):
        self.geom_modes = np.ascontiguousarray(geom_modes, dtype=np.uint32).reshape(-1, 3)
        self.geom_offset = np.ascontiguousarray(geom_offset, dtype=np.int64)
        self.geom = np.ascontiguousarray(geom, dtype=np.float32)
        self.field_modes = np.ascontiguousarray(field_modes, dtype=np.uint32).reshape(-1, 3)
        self.field_offset = np.ascontiguousarray(field_offset, dtype=np.int64)
        self.field = np.ascontiguousarray(field, dtype=np.float32)
        if self.field.size == 0:
            self.field = np.zeros(1, np.float32)
        if self.geom.size == 0:
            self.geom = np.zeros(1, np.float32)
        self.verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 8, 3)

    @property
    def n(self) -> int:
        return int(self.geom_modes.shape[0])

    def save(self, path):
        np.savez_compressed(path, geom_modes=self.geom_modes, geom_offset=self.geom_offset, geom=self.geom,
                            field_modes=self.field_modes, field_offset=self.field_offset, field=self.field,
                            verts=self.verts)

    @staticmethod
    def load(path) -> "SceneArrays":
        z = np.load(path)
        return SceneArrays(z["geom_modes"], z["geom_offset"], z["geom"], z["field_modes"], z["field_offset"],
                           z["field"], z["verts"])


def synth_scene(nx, ny, nz, order_min, order_max, curve_amp, n_gauss, seed, threads: int = 0) -> SceneArrays:
    """The seeded synthetic scene that ho_generate_synthetic describes, built
    by the oracle's own generator (oracle/horender_synth.cpp): no product
    library is loaded."""
    prm = _SynthParams(int(nx), int(ny), int(nz), int(order_min), int(order_max), float(curve_amp), int(n_gauss),
                       int(seed))
    ne, gl, fl = C.c_int64(), C.c_int64(), C.c_int64()
    if lib().hor_synth_sizes(C.byref(prm), C.byref(ne), C.byref(gl), C.byref(fl)) != 0:
        raise ValueError("invalid synthetic scene parameters")
    n = ne.value
    verts = np.zeros((n, 8, 3), np.float32)
    gm = np.zeros((n, 3), np.uint32)
    go = np.zeros(n, np.int64)
    g = np.zeros(gl.value, np.float32)
    fm = np.zeros((n, 3), np.uint32)
    fo = np.zeros(n, np.int64)
    f = np.zeros(fl.value, np.float32)
    rc = lib().hor_synth_fill(C.byref(prm), int(threads), _p(verts), _p(gm), _p(go), _p(g), _p(fm), _p(fo), _p(f))
    if rc != 0:
        raise RuntimeError(f"hor_synth_fill failed ({rc})")
    return SceneArrays(gm, go, g, fm, fo, f, verts)


class OracleScene:
    def __init__(self, arrs: SceneArrays):
        self.arrs = arrs
        d = _SceneDesc(arrs.n, _p(arrs.geom_modes).value, _p(arrs.geom_offset).value, _p(arrs.geom).value,
                       _p(arrs.field_modes).value, _p(arrs.field_offset).value, _p(arrs.field).value,
                       _p(arrs.verts).value)
        self.h = lib().hor_scene_create(C.byref(d))

    def __del__(self):
        if getattr(self, "h", None):
            lib().hor_scene_destroy(self.h)
            self.h = None

    def boxes(self, precision=64) -> np.ndarray:
        out = np.zeros((self.arrs.n, 6), np.float64)
        lib().hor_scene_boxes(self.h, precision, _p(out))
        return out

    def trace(self, rays: np.ndarray, iso: float, iso_on: bool = True, precision: int = 64,
              threads: int | None = None):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = np.zeros(rays.shape[0], HIT_DTYPE)
        cnt = _Counters()
        nt = threads or os.cpu_count() or 1
        lib().hor_trace(self.h, precision, _p(rays), rays.shape[0], float(iso), int(iso_on), nt, _p(out),
                        C.byref(cnt))
        return out, {k: getattr(cnt, k) for k, _ in _Counters._fields_}

    def polish(self, rays, hits, iso, threads=None):
        """The judge's FP64 polish of given hits (HIT_DTYPE, oracle or product
        hits converted): each hit's defining equations solved to convergence
        from its own (t, xi). Returns a copy; pad = 1 where it converged."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        out = np.zeros(rays.shape[0], HIT_DTYPE)
        for k in ("t", "elem", "face", "kind", "xi", "n", "u"):
            out[k] = hits[k]
        nt = threads or os.cpu_count() or 1
        lib().hor_polish(self.h, _p(rays), rays.shape[0], float(iso), _p(out), nt)
        return out

    def trace_replay(self, rays, iso, iso_on, order, order_n, precision=32):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        order = np.ascontiguousarray(order, np.int32)
        order_n = np.ascontiguousarray(order_n, np.int32)
        out = np.zeros(rays.shape[0], HIT_DTYPE)
        lib().hor_trace_replay(self.h, precision, _p(rays), rays.shape[0], float(iso), int(iso_on), _p(order),
                               order.shape[1], _p(order_n), _p(out))
        return out

    def map_point(self, elem, xi, precision=64):
        xi = np.ascontiguousarray(xi, np.float64).reshape(-1, 3)
        out = np.zeros_like(xi)
        lib().hor_map_point(self.h, precision, elem, _p(xi), xi.shape[0], _p(out))
        return out

    def eval_point(self, elem, xi, precision=64):
        xi = np.ascontiguousarray(xi, np.float64).reshape(-1, 3)
        out = np.zeros((xi.shape[0], 13))
        lib().hor_eval_point(self.h, precision, elem, _p(xi), xi.shape[0], _p(out))
        return out

    def inverse_map(self, elem, x, precision=64):
        x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        out = np.zeros((x.shape[0], 4))
        lib().hor_inverse_map(self.h, precision, elem, _p(x), x.shape[0], _p(out))
        return out

    def find_iso(self, elem, rays, seg, iso, precision=64):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        seg = np.ascontiguousarray(seg, np.float64).reshape(-1, 2)
        out = np.zeros((rays.shape[0], 8))
        lib().hor_find_iso(self.h, precision, elem, _p(rays), _p(seg), rays.shape[0], float(iso), _p(out))
        return out

    def hit_hex(self, elem, rays, seg, precision=64):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        seg = np.ascontiguousarray(seg, np.float64).reshape(-1, 2)
        out = np.zeros((rays.shape[0], 6))
        lib().hor_hit_hex(self.h, precision, elem, _p(rays), _p(seg), rays.shape[0], _p(out))
        return out


PRIM_PRISM, PRIM_QUAD, PRIM_TRI = 0, 1, 2
NVERTS = {PRIM_PRISM: 6, PRIM_QUAD: 4, PRIM_TRI: 3}


class PrimArrays:
    """Prisms, quads and curved triangles as one list (kind-major: all prisms,
    then quads, then triangles, as the product stores them): kind (n), vertices
    (n x 6 x 3, unused rows zero), geometry/field modes (n x 3), offsets
    (-1 = linear geometry / no field) into flat fp32 pools; a geometry entry
    is the x, y and z blocks back to back."""

    def __init__(self, kind, verts, geom_modes, geom_offset, geom, field_modes, field_offset, field):
        self.kind = np.ascontiguousarray(kind, np.int32)
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 6, 3)
        self.geom_modes = np.ascontiguousarray(geom_modes, np.uint32).reshape(-1, 3)
        self.geom_offset = np.ascontiguousarray(geom_offset, np.int64)
        self.geom = np.ascontiguousarray(geom, np.float32)
        self.field_modes = np.ascontiguousarray(field_modes, np.uint32).reshape(-1, 3)
        self.field_offset = np.ascontiguousarray(field_offset, np.int64)
        self.field = np.ascontiguousarray(field, np.float32)

    @property
    def n(self) -> int:
        return int(self.kind.shape[0])

    def of_kind(self, k):
        """(vertices n_k x nv x 3, geometry modes, offsets, field modes, offsets) of one kind."""
        m = self.kind == k
        return (self.verts[m][:, :NVERTS[k]], self.geom_modes[m], self.geom_offset[m], self.field_modes[m],
                self.field_offset[m])


class OraclePrims:
    def __init__(self, arrs: PrimArrays):
        self.arrs = arrs
        g = arrs.geom if arrs.geom.size else np.zeros(1, np.float32)
        f = arrs.field if arrs.field.size else np.zeros(1, np.float32)
        self._keep = (g, f)
        d = _PrimsDesc(arrs.n, _p(arrs.kind).value, _p(arrs.verts).value, _p(arrs.geom_modes).value,
                       _p(arrs.geom_offset).value, _p(g).value, arrs.geom.size, _p(arrs.field_modes).value,
                       _p(arrs.field_offset).value, _p(f).value, arrs.field.size)
        self.h = lib().hor_prims_create(C.byref(d))

    def __del__(self):
        if getattr(self, "h", None):
            lib().hor_prims_destroy(self.h)
            self.h = None

    def boxes(self, precision=32) -> np.ndarray:
        out = np.zeros((self.arrs.n, 6))
        lib().hor_prims_boxes(self.h, precision, _p(out))
        return out

    def intersect(self, prim, rays, seg, precision=32):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        seg = np.ascontiguousarray(seg, np.float64).reshape(-1, 2)
        out = np.zeros((rays.shape[0], 5))
        assert lib().hor_prims_intersect(self.h, precision, prim, _p(rays), rays.shape[0], _p(seg), _p(out)) == 0
        return out

    def map(self, prim, xi, precision=64):
        xi = np.ascontiguousarray(xi, np.float64).reshape(-1, 3)
        out = np.zeros_like(xi)
        lib().hor_prims_map(self.h, precision, prim, _p(xi), xi.shape[0], _p(out))
        return out

    def trace(self, rays, hex_hits=None, precision=32, threads=None):
        """The primitive pass after the hexahedra: hex_hits (HIT_DTYPE, or
        None = all miss) is each ray's hexahedron answer; returns the merged hits."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        io = np.zeros(rays.shape[0], HIT_DTYPE) if hex_hits is None else np.array(hex_hits, HIT_DTYPE, copy=True)
        if hex_hits is None:
            io["elem"] = -1
            io["face"] = -1
        lib().hor_prims_trace(self.h, precision, _p(rays), rays.shape[0], _p(io), threads or os.cpu_count() or 1)
        return io


def basis(nmodes: int, x: float, precision=64) -> np.ndarray:
    out = np.zeros((nmodes, 2))
    lib().hor_basis(precision, nmodes, float(x), _p(out))
    return out


def camera_rays(lookfrom, lookat, vup, vfov, W, H) -> np.ndarray:
    f = np.asarray(lookfrom, np.float32)
    a = np.asarray(lookat, np.float32)
    u = np.asarray(vup, np.float32)
    out = np.zeros((H * W, 6), np.float32)
    lib().hor_camera_rays(_p(f), _p(a), _p(u), float(vfov), W, H, _p(out))
    return out


def shade(rays: np.ndarray, hits: np.ndarray) -> np.ndarray:
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    hits = np.ascontiguousarray(hits, HIT_DTYPE)
    out = np.zeros((rays.shape[0], 3), np.uint8)
    lib().hor_shade(_p(rays), _p(hits), rays.shape[0], _p(out))
    return out


# ---------------------------------------------------------------------------
# reference shim (only where oracle/_ref was built from the reference sources)
# ---------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    return REF_SO.exists()


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(str(REF_SO))
        vp, i32, i64, f32 = C.c_void_p, C.c_int, C.c_int64, C.c_float
        L.ref_scene_create.restype = vp
        L.ref_scene_create.argtypes = [i32, vp, vp, vp, i64, vp, vp, vp, i64, vp]
        L.ref_scene_load.restype = vp
        L.ref_scene_load.argtypes = [C.c_char_p, C.c_char_p]
        L.ref_prim_intersect.argtypes = [i32, vp, vp, vp, vp, vp, vp, i64, vp, vp, vp]
        L.ref_vtu_prim_verts.argtypes = [C.c_char_p, vp, vp]
        L.ref_scene_load_vtu.restype = vp
        L.ref_scene_load_vtu.argtypes = [C.c_char_p, vp]
        L.ref_scene_destroy.argtypes = [vp]
        L.ref_scene_count.argtypes = [vp]
        L.ref_scene_elem.argtypes = [vp, i32, vp, vp, vp, vp]
        L.ref_scene_geom.restype = i64
        L.ref_scene_geom.argtypes = [vp, vp]
        L.ref_scene_field.restype = i64
        L.ref_scene_field.argtypes = [vp, vp]
        L.ref_basis.argtypes = [C.c_uint, f32, vp]
        L.ref_box.argtypes = [vp, i32, i32, vp]
        L.ref_map_point.argtypes = [vp, i32, vp, i64, vp]
        L.ref_eval_point.argtypes = [vp, i32, vp, i64, vp]
        L.ref_inverse_map.argtypes = [vp, i32, vp, i64, vp]
        L.ref_find_iso.argtypes = [vp, i32, vp, vp, i64, f32, vp]
        L.ref_hit_hex.argtypes = [vp, i32, vp, vp, i64, vp]
        L.ref_trace.argtypes = [vp, vp, i64, f32, vp]
        L.ref_trace_order.argtypes = [vp, vp, i64, f32, vp, vp, i32, vp]
        L.ref_trace_order_iso.argtypes = [vp, vp, i64, f32, i32, vp, vp, i32, vp]
        _ref = L
    return _ref


class RefScene:
    def __init__(self, arrs: SceneArrays | None = None, xml: str | None = None, fld: str | None = None,
                 vtu: str | None = None):
        L = ref()
        if vtu is not None:
            # hexahedra, prisms and quads the reference loader added
            self.vtu_counts = np.zeros(3, np.int64)
            self.h = L.ref_scene_load_vtu(vtu.encode(), _p(self.vtu_counts))
            if not self.h:
                raise RuntimeError("reference loader failed")
            self.vtu_prisms = np.zeros((int(self.vtu_counts[1]), 6, 3), np.float32)
            self.vtu_quads = np.zeros((int(self.vtu_counts[2]), 4, 3), np.float32)
            L.ref_vtu_prim_verts(vtu.encode(), _p(self.vtu_prisms), _p(self.vtu_quads))
        elif xml is not None:
            self.h = L.ref_scene_load(xml.encode(), fld.encode())
            if not self.h:
                raise RuntimeError("reference loader failed")
        else:
            self.arrs = arrs
            self.h = L.ref_scene_create(arrs.n, _p(arrs.geom_modes), _p(arrs.geom_offset), _p(arrs.geom),
                                        arrs.geom.size, _p(arrs.field_modes), _p(arrs.field_offset),
                                        _p(arrs.field), arrs.field.size, _p(arrs.verts))

    def __del__(self):
        if getattr(self, "h", None):
            ref().ref_scene_destroy(self.h)
            self.h = None

    def arrays(self) -> SceneArrays:
        L = ref()
        n = L.ref_scene_count(self.h)
        gm = np.zeros((n, 3), np.uint32)
        fm = np.zeros((n, 3), np.uint32)
        go = np.zeros(n, np.int64)
        fo = np.zeros(n, np.int64)
        verts = np.zeros((n, 8, 3), np.float32)
        modes6 = np.zeros(6, np.uint32)
        offs = np.zeros(2, np.int64)
        v24 = np.zeros(24, np.float32)
        box = np.zeros(6, np.float32)
        for i in range(n):
            L.ref_scene_elem(self.h, i, _p(modes6), _p(offs), _p(v24), _p(box))
            gm[i] = modes6[:3]
            fm[i] = modes6[3:]
            go[i], fo[i] = offs
            verts[i] = v24.reshape(8, 3)
        ng = L.ref_scene_geom(self.h, None)
        geom = np.zeros(ng, np.float32)
        L.ref_scene_geom(self.h, _p(geom))
        nf = L.ref_scene_field(self.h, None)
        field = np.zeros(nf, np.float32)
        L.ref_scene_field(self.h, _p(field))
        return SceneArrays(gm, go, geom, fm, fo, field, verts)

    def box(self, elem, samples):
        out = np.zeros(6, np.float32)
        ref().ref_box(self.h, elem, samples, _p(out))
        return out

    def map_point(self, elem, xi):
        xi = np.ascontiguousarray(xi, np.float32).reshape(-1, 3)
        out = np.zeros_like(xi)
        ref().ref_map_point(self.h, elem, _p(xi), xi.shape[0], _p(out))
        return out

    def eval_point(self, elem, xi):
        xi = np.ascontiguousarray(xi, np.float32).reshape(-1, 3)
        out = np.zeros((xi.shape[0], 13), np.float32)
        ref().ref_eval_point(self.h, elem, _p(xi), xi.shape[0], _p(out))
        return out

    def inverse_map(self, elem, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        out = np.zeros((x.shape[0], 4), np.float32)
        ref().ref_inverse_map(self.h, elem, _p(x), x.shape[0], _p(out))
        return out

    def find_iso(self, elem, rays, seg, iso):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        seg = np.ascontiguousarray(seg, np.float32).reshape(-1, 2)
        out = np.zeros((rays.shape[0], 8), np.float32)
        ref().ref_find_iso(self.h, elem, _p(rays), _p(seg), rays.shape[0], float(iso), _p(out))
        return out

    def hit_hex(self, elem, rays, seg):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        seg = np.ascontiguousarray(seg, np.float32).reshape(-1, 2)
        out = np.zeros((rays.shape[0], 6), np.float32)
        ref().ref_hit_hex(self.h, elem, _p(rays), _p(seg), rays.shape[0], _p(out))
        return out

    def trace(self, rays, iso, order_cap: int = 0, iso_always: bool = False):
        """Reference traversal; returns (n x 12 results) or, with order_cap > 0,
        (results, visit order n x order_cap, visit counts). iso_always: call
        FindIsosurfaceOnRayHex at every isovalue, 0.0 included (the renderer
        turns the isosurface off at 0)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.zeros((rays.shape[0], 12), np.float32)
        order = np.zeros((rays.shape[0], max(order_cap, 1)), np.int32)
        cnt = np.zeros(rays.shape[0], np.int32)
        ref().ref_trace_order_iso(self.h, _p(rays), rays.shape[0], float(iso), int(iso_always), _p(out),
                                  _p(order) if order_cap > 0 else None, order_cap, _p(cnt))
        if order_cap <= 0:
            return out
        return out, order, cnt


def ref_prim_intersect(arrs: PrimArrays, prim: int, rays, seg):
    """The reference's own box and IntersectRayWith* for primitive `prim` of
    arrs: (box (6,), results n x 5 = hit, t, r, s, t-coordinate)."""
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
    seg = np.ascontiguousarray(seg, np.float64).reshape(-1, 2)
    k = int(arrs.kind[prim])
    verts = np.ascontiguousarray(arrs.verts[prim], np.float32)
    gm = np.ascontiguousarray(arrs.geom_modes[prim], np.uint32)
    ptrs = [None, None, None]
    keep = []
    if arrs.geom_offset[prim] >= 0:
        from_ = int(arrs.geom_offset[prim])
        m = [int(v) for v in gm]
        if k == PRIM_QUAD:
            blk = m[0] * m[1]
        else:
            top = m[2] if k == PRIM_PRISM else m[1]
            blk = sum(max(top - i, 0) for i in range(m[0])) * (m[1] if k == PRIM_PRISM else 1)
        for a in range(3):
            b = np.ascontiguousarray(arrs.geom[from_ + a * blk: from_ + (a + 1) * blk], np.float32)
            keep.append(b)
            ptrs[a] = _p(b)
    box = np.zeros(6, np.float32)
    out = np.zeros((rays.shape[0], 5))
    ref().ref_prim_intersect(k, _p(verts), _p(gm), ptrs[0], ptrs[1], ptrs[2], _p(rays), rays.shape[0], _p(seg),
                             _p(box), _p(out))
    return box, out


def ref_basis(nmodes: int, x: float) -> np.ndarray:
    out = np.zeros((nmodes, 2), np.float32)
    ref().ref_basis(nmodes, float(x), _p(out))
    return out
