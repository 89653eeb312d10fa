"""Seeded synthetic scenes of prisms, quads and curved triangles (host-side
generator for tests and the benchmark; the kernels never see it).

High-order geometry is a least-squares fit, in the primitive's own modal
basis (Modified-A x Modified-A x Modified-B for the prism, A x A for the
quad, A x B for the triangle, as FEM-AABB/fem/PrismElement.cu, QuadElement.cu
and TriElement.cu evaluate them), of its linear map plus a smooth bump, so
the coefficients are ordinary fp32 numbers.

Vertex conventions (the reference's linear maps): prism vertices 0-3 are the
quad at t = -1 in the order (-,-), (+,-), (+,+), (-,+) of (r, s) and 4, 5 the
top edge at s = -1, +1; quad vertex v sits at r = +-1 by bit 0, s = +-1 by
bit 1; triangle vertices at barycentric (0,0), (1,0), (0,1)."""
from __future__ import annotations

from functools import lru_cache

import numpy as np

PRISM, QUAD, TRI = 0, 1, 2
NVERTS = {PRISM: 6, QUAD: 4, TRI: 3}


def jacobi(n, a, b, x):
    x = np.asarray(x, np.float64)
    if n == 0:
        return np.ones_like(x)
    p0, p1 = np.ones_like(x), 0.5 * ((2 + a + b) * x + (a - b))
    for k in range(2, n + 1):
        s = 2 * k + a + b
        p0, p1 = p1, ((s - 1) * (s * (s - 2) * x + (a * a - b * b)) * p1 - 2 * (k + a - 1) * (k + b - 1) * s * p0) / (
            2 * k * (k + a + b) * (s - 2))
    return p1


def mod_a(i, x):
    if i == 0:
        return 0.5 * (1 - x)
    if i == 1:
        return 0.5 * (1 + x)
    return 0.25 * (1 - x * x) * jacobi(i - 2, 1.0, 1.0, x)


def mod_b(i, j, x):
    if i == 0:
        return mod_a(j, x)
    v = (0.5 * (1 - x)) ** i
    if j == 0:
        return v
    return v * 0.5 * (1 + x) * jacobi(j - 1, 2.0 * i - 1.0, 1.0, x)


def basis_matrix(kind, m, pts):
    """Modal basis values at pts (n x 3), columns in the coefficient order."""
    cols = []
    if kind == PRISM:
        for i in range(m[0]):
            for j in range(m[1]):
                for k in range(max(m[2] - i, 0)):
                    cols.append(mod_a(i, pts[:, 0]) * mod_a(j, pts[:, 1]) * mod_b(i, k, pts[:, 2]))
    elif kind == QUAD:
        for j in range(m[1]):
            for i in range(m[0]):
                cols.append(mod_a(i, pts[:, 0]) * mod_a(j, pts[:, 1]))
    else:
        for i in range(m[0]):
            for j in range(max(m[1] - i, 0)):
                cols.append(mod_a(i, pts[:, 0]) * mod_b(i, j, pts[:, 1]))
    return np.stack(cols, 1)


def block_size(kind, m):
    return int(basis_matrix(kind, m, np.zeros((1, 3))).shape[1])


@lru_cache(maxsize=None)
def _fit_operator(kind, m):
    pts = np.random.default_rng(1234).uniform(-1, 1, (600, 3))
    return pts, np.linalg.pinv(basis_matrix(kind, m, pts))


def linear_map(kind, verts, pts):
    v = np.asarray(verts, np.float64)
    if kind == PRISM:
        r, s, t = pts[:, 0:1], pts[:, 1:2], pts[:, 2:3]
        w = [0.125 * (1 - r) * (1 - s) * (1 - t), 0.125 * (1 + r) * (1 - s) * (1 - t),
             0.125 * (1 + r) * (1 + s) * (1 - t), 0.125 * (1 - r) * (1 + s) * (1 - t),
             0.25 * (1 - s) * (1 + t), 0.25 * (1 + s) * (1 + t)]
    elif kind == QUAD:
        r, s = pts[:, 0:1], pts[:, 1:2]
        w = [0.25 * (1 + (1 if q & 1 else -1) * r) * (1 + (1 if q & 2 else -1) * s) for q in range(4)]
    else:
        # (r, s) as the collapsed coordinates the modal triangle uses
        e1, e2 = pts[:, 0:1], pts[:, 1:2]
        u = 0.5 * (1 + e1) * 0.5 * (1 - e2)
        vv = 0.5 * (1 + e2)
        w = [1 - u - vv, u, vv]
    return sum(wi * v[i] for i, wi in enumerate(w))


def fit_geometry(kind, verts, m, amp, direction):
    """Coefficients (x, y, z blocks) of the linear map plus a smooth bump."""
    pts, pinv = _fit_operator(kind, tuple(int(v) for v in m))
    target = linear_map(kind, verts, pts)
    c = np.asarray(direction, np.float64)
    target = target + amp * np.sin(np.pi * 0.5 * (pts[:, 0:1] + 1)) * np.sin(np.pi * 0.5 * (pts[:, 1:2] + 1)) * c
    return (pinv @ target).T.reshape(-1).astype(np.float32)


class PrimSet:
    """Primitives as one kind-major list (all prisms, then quads, then
    triangles): kind (n), vertices (n x 6 x 3, unused rows zero), modes
    (n x 3), offsets (-1 = linear geometry / no field) into flat fp32 pools."""

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


class Builder:
    """Collects primitives kind by kind; build() returns them kind-major."""

    def __init__(self):
        self.items = {0: [], 1: [], 2: []}

    def add(self, kind, verts, geom=None, gm=(0, 0, 0), field=None, fm=(0, 0, 0)):
        v = np.zeros((6, 3), np.float32)
        v[:NVERTS[kind]] = np.asarray(verts, np.float32)
        self.items[kind].append((v, geom, tuple(gm), field, tuple(fm)))

    def build(self) -> PrimSet:
        kind, verts, gm, go, fm, fo = [], [], [], [], [], []
        geom, field = [], []
        ng = nf = 0
        for k in (0, 1, 2):
            for v, g, m, f, fmm in self.items[k]:
                kind.append(k)
                verts.append(v)
                gm.append(m if g is not None else (0, 0, 0))
                go.append(ng if g is not None else -1)
                if g is not None:
                    geom.append(g)
                    ng += g.size
                fm.append(fmm if f is not None else (0, 0, 0))
                fo.append(nf if f is not None else -1)
                if f is not None:
                    field.append(f)
                    nf += f.size
        cat = lambda xs: np.concatenate(xs).astype(np.float32) if xs else np.zeros(0, np.float32)
        return PrimSet(np.array(kind, np.int32), np.array(verts, np.float32).reshape(-1, 6, 3),
                       np.array(gm, np.uint32).reshape(-1, 3), np.array(go, np.int64), cat(geom),
                       np.array(fm, np.uint32).reshape(-1, 3), np.array(fo, np.int64), cat(field))


def tent(x0, y0, z0, w, d, h):
    """Prism lying on its quad: base (x0..x0+w) x (z0..z0+d) at y0, ridge at height h."""
    return [(x0, y0, z0), (x0 + w, y0, z0), (x0 + w, y0, z0 + d), (x0, y0, z0 + d),
            (x0 + 0.5 * w, y0 + h, z0), (x0 + 0.5 * w, y0 + h, z0 + d)]


def mixed_scene(seed=0, n_side=4, curved=True) -> PrimSet:
    """Tents (prisms) on a floor of quads, a wall of triangles behind, in
    [0, 1]^3; about half of each kind curved, most with a field."""
    rng = np.random.default_rng(seed)
    b = Builder()
    cell = 1.0 / n_side

    def maybe(kind, verts, m, fm):
        geom = None
        if curved and rng.random() < 0.5:
            geom = fit_geometry(kind, verts, m, 0.15 * cell, rng.normal(size=3) / 2)
        field = rng.normal(size=block_size(kind, fm)).astype(np.float32) * 0.3 if rng.random() < 0.7 else None
        b.add(kind, verts, geom, m if geom is not None else (0, 0, 0), field, fm)

    for i in range(n_side):
        for k in range(n_side):
            if (i + k) % 2 == 0:
                verts = tent(i * cell + 0.1 * cell, 0.0, k * cell + 0.1 * cell, 0.8 * cell, 0.8 * cell,
                             0.6 * cell * (0.7 + 0.6 * rng.random()))
                maybe(PRISM, verts, (3, 3, 3), (3, 3, 3))
    for i in range(n_side):
        for k in range(n_side):
            x0, z0 = i * cell, k * cell
            verts = [(x0, 0.0, z0), (x0 + cell, 0.0, z0), (x0, 0.0, z0 + cell), (x0 + cell, 0.0, z0 + cell)]
            verts = np.array(verts) + np.array([0, -0.02, 0]) * rng.random()
            maybe(QUAD, verts, (4, 4, 0), (3, 3, 0))
    for i in range(n_side):
        for j in range(n_side):
            x0, y0 = i * cell, j * cell
            lo = [(x0, y0, 0.0), (x0 + cell, y0, 0.0), (x0, y0 + cell, 0.0)]
            hi = [(x0 + cell, y0 + cell, 0.0), (x0, y0 + cell, 0.0), (x0 + cell, y0, 0.0)]
            maybe(TRI, lo, (4, 4, 0), (3, 3, 0))
            maybe(TRI, hi, (4, 4, 0), (3, 3, 0))
    return b.build()
