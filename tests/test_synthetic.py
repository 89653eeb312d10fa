"""Properties of the seeded synthetic scenes (host generator), checked with
the FP64 oracle: corners, cube boundary, conforming shared faces, field
continuity, determinism and the order range of mixed-order scenes."""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import oracle_bind as ob
from conftest import scene_arrays_from_ctx


@pytest.fixture(scope="module")
def scene(oracle):
    ctx = hr.Context(0)
    ctx.generate_synthetic(3, 3, 3, 4, 4, 0.1, 8, 7)
    arrs = scene_arrays_from_ctx(ctx)
    ctx.close()
    return arrs, ob.OracleScene(arrs)


CORNERS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1],
                    [-1, 1, 1]], float)


def eid(kx, ky, kz, n=3):
    return (kz * n + ky) * n + kx


def test_corners_match_geometry(scene):
    arrs, osc = scene
    for e in range(arrs.n):
        assert np.abs(osc.map_point(e, CORNERS) - arrs.verts[e]).max() < 2e-6


def test_boundary_faces_stay_on_the_cube(scene):
    arrs, osc = scene
    rng = np.random.default_rng(1)
    st = rng.uniform(-1, 1, (64, 2))
    xi = np.c_[-np.ones(64), st]
    for ky in range(3):
        for kz in range(3):
            x = osc.map_point(eid(0, ky, kz), xi)
            assert np.abs(x[:, 0]).max() < 2e-6


def test_shared_faces_conform(scene):
    arrs, osc = scene
    rng = np.random.default_rng(2)
    st = rng.uniform(-1, 1, (64, 2))
    for kx in range(2):
        a, b = eid(kx, 1, 1), eid(kx + 1, 1, 1)
        xa = osc.map_point(a, np.c_[np.ones(64), st])
        xb = osc.map_point(b, np.c_[-np.ones(64), st])
        assert np.abs(xa - xb).max() < 2e-6
        ua = osc.eval_point(a, np.c_[np.ones(64), st])[:, 9]
        ub = osc.eval_point(b, np.c_[-np.ones(64), st])[:, 9]
        assert np.abs(ua - ub).max() < 2e-6


def test_elements_are_curved_and_valid(scene):
    arrs, osc = scene
    rng = np.random.default_rng(3)
    xi = rng.uniform(-1, 1, (64, 3))
    e = eid(1, 1, 1)
    J = osc.eval_point(e, xi)[:, :9].reshape(-1, 3, 3)
    assert (np.linalg.det(J) > 0).all()
    # curved: the map differs from the trilinear map through its corners
    p = np.array([0.3, -0.4, 0.2])
    w = [np.prod([(1 + c * q) / 2 for c, q in zip(CORNERS[v], p)]) for v in range(8)]
    tri = np.einsum("v,vc->c", np.array(w), arrs.verts[e].astype(np.float64))
    assert np.abs(osc.map_point(e, p[None])[0] - tri).max() > 1e-4


def test_deterministic_and_order_range():
    def gen():
        with hr.Context(0) as ctx:
            ctx.generate_synthetic(4, 4, 4, 2, 8, 0.1, 16, 3)
            return ctx.get_scene()

    a, b = gen(), gen()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    m = a["geom_modes"][:, 0]
    assert m.min() >= 3 and m.max() <= 9 and len(np.unique(m)) >= 5


@pytest.mark.parametrize("synth", [dict(nx=3, ny=2, nz=4, order_min=2, order_max=8, curve_amp=0.1, n_gauss=16, seed=9),
                                   hr.WORKLOADS["hex4_p4"].synth()])
def test_oracle_generator_equals_library(oracle, synth):
    """The oracle's own generator (oracle/horender_synth.cpp), which the
    benchmark's CPU arm uses so that it loads no product library, makes the
    library's scene: same layout, corners and coefficients (identical on a
    host compiler that does not fuse multiply-adds; within FP32 rounding of
    the FP64 fit otherwise)."""
    a = ob.synth_scene(**synth)
    ctx = hr.Context(0)
    ctx.generate_synthetic(**synth)
    s = ctx.get_scene()
    ctx.close()
    assert np.array_equal(a.geom_modes.reshape(-1), s["geom_modes"].reshape(-1))
    assert np.array_equal(a.geom_offset, s["geom_offsets"]) and np.array_equal(a.field_offset, s["field_offsets"])
    assert np.array_equal(a.verts.reshape(-1), s["corners"].reshape(-1))
    for x, y in ((a.geom, s["geom"]), (a.field, s["field"])):
        assert x.shape == y.shape
        assert np.abs(x - y).max() <= 1e-6 * max(1.0, np.abs(y).max())
        assert (x == y).mean() > 0.99
