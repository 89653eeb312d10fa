"""Seeded prism / quad / curved-triangle scenes for the primitive tests
(test infrastructure). High-order geometry is a least-squares fit, in the
primitive's own modal basis, of its linear map plus a smooth bump, so the
coefficients are ordinary fp32 numbers that the reference, the oracle and the
product all read the same way.

Vertex conventions (the reference's linear maps): prism vertices 0-3 are the
quad at t = -1 in the order (-,-), (+,-), (+,+), (-,+) of (r, s) and 4, 5 the
top edge at s = -1, +1; quad vertex v sits at r = +-1 by bit 0, s = +-1 by
bit 1; triangle vertices at barycentric (0,0), (1,0), (0,1)."""
from __future__ import annotations

import numpy as np

import oracle_bind as ob


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
    cols = []
    if kind == ob.PRIM_PRISM:
        for i in range(m[0]):
            for j in range(m[1]):
                for k in range(max(m[2] - i, 0)):
                    cols.append(mod_a(i, pts[:, 0]) * mod_a(j, pts[:, 1]) * mod_b(i, k, pts[:, 2]))
    elif kind == ob.PRIM_QUAD:
        for j in range(m[1]):
            for i in range(m[0]):
                cols.append(mod_a(i, pts[:, 0]) * mod_a(j, pts[:, 1]))
    else:
        for i in range(m[0]):
            for j in range(max(m[1] - i, 0)):
                cols.append(mod_a(i, pts[:, 0]) * mod_b(i, j, pts[:, 1]))
    return np.stack(cols, 1)


def linear_map(kind, verts, pts):
    v = np.asarray(verts, np.float64)
    if kind == ob.PRIM_PRISM:
        r, s, t = pts[:, 0:1], pts[:, 1:2], pts[:, 2:3]
        w = [0.125 * (1 - r) * (1 - s) * (1 - t), 0.125 * (1 + r) * (1 - s) * (1 - t),
             0.125 * (1 + r) * (1 + s) * (1 - t), 0.125 * (1 - r) * (1 + s) * (1 - t),
             0.25 * (1 - s) * (1 + t), 0.25 * (1 + s) * (1 + t)]
    elif kind == ob.PRIM_QUAD:
        r, s = pts[:, 0:1], pts[:, 1:2]
        w = [0.25 * (1 + (1 if q & 1 else -1) * r) * (1 + (1 if q & 2 else -1) * s) for q in range(4)]
    else:
        # (r, s) as the collapsed coordinates the modal triangle uses
        e1, e2 = pts[:, 0:1], pts[:, 1:2]
        u = 0.5 * (1 + e1) * 0.5 * (1 - e2)
        vv = 0.5 * (1 + e2)
        w = [1 - u - vv, u, vv]
    return sum(wi * v[i] for i, wi in enumerate(w))


def fit_geometry(kind, verts, m, bump, rng):
    """Coefficients (x, y, z blocks) of the linear map plus a smooth bump."""
    n = 600
    pts = rng.uniform(-1, 1, (n, 3))
    target = linear_map(kind, verts, pts)
    c = np.asarray(bump["dir"], np.float64)
    target = target + bump["amp"] * np.sin(np.pi * 0.5 * (pts[:, 0:1] + 1)) * np.sin(np.pi * 0.5 * (pts[:, 1:2] + 1)) * c
    B = basis_matrix(kind, m, pts)
    coef, *_ = np.linalg.lstsq(B, target, rcond=None)
    return coef.T.reshape(-1).astype(np.float32)  # x block, y block, z block


def block_size(kind, m):
    return int(basis_matrix(kind, m, np.zeros((1, 3))).shape[1])


class Builder:
    """Collects primitives kind by kind; arrays() returns them kind-major."""

    def __init__(self):
        self.items = {0: [], 1: [], 2: []}

    def add(self, kind, verts, geom=None, gm=(0, 0, 0), field=None, fm=(0, 0, 0)):
        v = np.zeros((6, 3), np.float32)
        v[:ob.NVERTS[kind]] = np.asarray(verts, np.float32)
        self.items[kind].append((v, geom, tuple(gm), field, tuple(fm)))

    def arrays(self) -> ob.PrimArrays:
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
        return ob.PrimArrays(np.array(kind, np.int32), np.array(verts, np.float32).reshape(-1, 6, 3),
                             np.array(gm, np.uint32).reshape(-1, 3), np.array(go, np.int64), cat(geom),
                             np.array(fm, np.uint32).reshape(-1, 3), np.array(fo, np.int64), cat(field))


def tent(x0, y0, z0, w, d, h):
    """Prism lying on its quad: base (x0..x0+w) x (z0..z0+d) at y0, ridge at height h."""
    return [(x0, y0, z0), (x0 + w, y0, z0), (x0 + w, y0, z0 + d), (x0, y0, z0 + d),
            (x0 + 0.5 * w, y0 + h, z0), (x0 + 0.5 * w, y0 + h, z0 + d)]


def mixed_scene(seed=0, n_side=4, curved=True):
    """Tents (prisms) on a floor of quads, a wall of triangles behind, in
    [0, 1]^3; about half of each kind curved, most with a field."""
    rng = np.random.default_rng(seed)
    b = Builder()
    cell = 1.0 / n_side

    def maybe(kind, verts, m, fm):
        geom = None
        if curved and rng.random() < 0.5:
            geom = fit_geometry(kind, verts, m, dict(amp=0.15 * cell, dir=rng.normal(size=3) / 2), rng)
        field = rng.normal(size=block_size(kind, fm)).astype(np.float32) * 0.3 if rng.random() < 0.7 else None
        b.add(kind, verts, geom, m if geom is not None else (0, 0, 0), field, fm)

    for i in range(n_side):
        for k in range(n_side):
            if (i + k) % 2 == 0:
                verts = tent(i * cell + 0.1 * cell, 0.0, k * cell + 0.1 * cell, 0.8 * cell, 0.8 * cell,
                             0.6 * cell * (0.7 + 0.6 * rng.random()))
                maybe(ob.PRIM_PRISM, verts, (3, 3, 3), (3, 3, 3))
    for i in range(n_side):
        for k in range(n_side):
            x0, z0 = i * cell, k * cell
            verts = [(x0, 0.0, z0), (x0 + cell, 0.0, z0), (x0, 0.0, z0 + cell), (x0 + cell, 0.0, z0 + cell)]
            verts = np.array(verts) + np.array([0, -0.02, 0]) * rng.random()
            maybe(ob.PRIM_QUAD, verts, (4, 4, 0), (3, 3, 0))
    for i in range(n_side):
        for j in range(n_side):
            x0, y0 = i * cell, j * cell
            lo = [(x0, y0, 0.0), (x0 + cell, y0, 0.0), (x0, y0 + cell, 0.0)]
            hi = [(x0 + cell, y0 + cell, 0.0), (x0, y0 + cell, 0.0), (x0 + cell, y0, 0.0)]
            maybe(ob.PRIM_TRI, lo, (4, 4, 0), (3, 3, 0))
            maybe(ob.PRIM_TRI, hi, (4, 4, 0), (3, 3, 0))
    return b.arrays()


def rays_at_boxes(arrs: ob.PrimArrays, boxes: np.ndarray, n_per: int, rng):
    """Per primitive n_per rays from outside its box towards random points in
    it, with segments [0.001, tmax] (tmax infinite for half of them, else
    somewhere along the box)."""
    out_r, out_s, owner = [], [], []
    for p in range(arrs.n):
        lo, hi = boxes[p, :3], boxes[p, 3:]
        c, ext = 0.5 * (lo + hi), np.maximum(hi - lo, 1e-3)
        tgt = lo[None] + rng.uniform(0, 1, (n_per, 3)) * ext[None]
        d = rng.normal(size=(n_per, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        o = tgt - d * (np.linalg.norm(ext) * 2 + 0.1)
        out_r.append(np.concatenate([o, d], 1))
        far = np.linalg.norm(ext) * 2 + 0.1 + rng.uniform(-1, 1, n_per) * np.linalg.norm(ext)
        tmax = np.where(rng.random(n_per) < 0.5, np.finfo(np.float32).max, far)
        out_s.append(np.stack([np.full(n_per, 0.001), tmax], 1))
        owner.append(np.full(n_per, p))
    return (np.concatenate(out_r).astype(np.float32), np.concatenate(out_s).astype(np.float64),
            np.concatenate(owner))
