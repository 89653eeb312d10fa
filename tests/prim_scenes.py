"""Primitive scenes for the tests (test infrastructure): the package's
seeded generator (prim_synth), wrapped as the oracle's PrimArrays, plus rays
aimed at each primitive's box."""
from __future__ import annotations

import numpy as np

import oracle_bind as ob
from prim_synth import (PRISM, QUAD, TRI, Builder, basis_matrix, block_size, fit_geometry, linear_map,  # noqa: F401
                        mod_a, mod_b, tent)
from prim_synth import mixed_scene as _mixed


def as_arrays(ps) -> ob.PrimArrays:
    return ob.PrimArrays(ps.kind, ps.verts, ps.geom_modes, ps.geom_offset, ps.geom, ps.field_modes, ps.field_offset,
                         ps.field)


def mixed_scene(seed=0, n_side=4, curved=True) -> ob.PrimArrays:
    return as_arrays(_mixed(seed, n_side, curved))


def shifted(arrs: ob.PrimArrays, dx: float) -> ob.PrimArrays:
    """The primitives moved by dx along x, curved geometry included: the x
    block holds the modal expansion of x, and a constant shift is carried by
    the vertex modes, whose values sum to 1 everywhere."""
    out = ob.PrimArrays(arrs.kind, arrs.verts + np.array([dx, 0, 0], np.float32), arrs.geom_modes,
                        arrs.geom_offset, arrs.geom.copy(), arrs.field_modes, arrs.field_offset, arrs.field)
    for p in range(arrs.n):
        if arrs.geom_offset[p] >= 0:
            blk = block_size(int(arrs.kind[p]), [int(v) for v in arrs.geom_modes[p]])
            o = int(arrs.geom_offset[p])
            B = basis_matrix(int(arrs.kind[p]), [int(v) for v in arrs.geom_modes[p]],
                             np.random.default_rng(0).uniform(-1, 1, (200, 3)))
            one, *_ = np.linalg.lstsq(B, np.ones(200), rcond=None)
            out.geom[o:o + blk] = (arrs.geom[o:o + blk] + dx * one).astype(np.float32)
    return out


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
