"""GPU kernels against the reference's own traced rays (golden fixtures made
from the reference build by tests/golden/make_golden.py), through the C ABI.

Identity. Per ray the GPU answer (kind, element, face) must equal the
reference's, or the ray must be explained; no other difference is allowed:
  order-dependent  the oracle replaying the reference's recorded visit order
                   returns the reference's answer, while the oracle in the
                   product's order (ascending padded-box entry) does not; the
                   product then answers like the oracle in its order (or
                   differs from it only by one of the classes below);
  tie / grazing / unstable   the classes of tests/parity.py: one surface
                   point claimed by two elements or faces, a grazing ray, or
                   a ray at a decision boundary of the reference algorithm
                   (its FP32 and FP64 answers differ, or the answer of the
                   oracle or of the product changes when the ray turns by at
                   most 4e-5 radians).
The counts of each class are printed.

Error. The reference's hits, polished in FP64 to the exact roots of their
own equations (the judge), against the GPU's hits where the identities
agree: t (the distance along the unit ray, so the error of the hit position)
within 1e-5 of the element size h, xi within 5e-5, u within 1e-5 — in every
solver mode (the FP64 polish of the final check). Hits of the same element
and face whose t differ by more than 1e-3 are different roots and count as
an identity difference.
"""
from __future__ import annotations

import numpy as np
import pytest

import horender as hr
import oracle_bind as ob
import parity
from conftest import GOLDEN, scene_arrays_from_ctx

pytestmark = pytest.mark.gpu

MODES = {"batched": hr.MODE_BATCHED, "learned": hr.MODE_LEARNED, "plain": hr.MODE_PLAIN}
POS_TOL = 1e-5   # of the element size
XI_TOL = parity.XI_TOL
U_TOL = 1e-5


def ref_hits(tr: np.ndarray) -> np.ndarray:
    """The reference's trace rows (kind, elem, face, t, xi, n, material, pad)
    as oracle hits."""
    h = np.zeros(tr.shape[0], ob.HIT_DTYPE)
    h["kind"] = tr[:, 0].astype(int)
    h["elem"] = tr[:, 1].astype(int)
    h["face"] = tr[:, 2].astype(int)
    h["t"] = tr[:, 3]
    h["xi"] = tr[:, 4:7]
    h["n"] = tr[:, 7:10]
    return h


def iso_tag(iso):
    return ("m" if iso < 0 else "p") + f"{abs(iso):.1f}".replace(".", "")


@pytest.fixture(scope="module", params=["hex32_p6", "hex64_p5"])
def golden(request):
    name = request.param
    z = np.load(GOLDEN / f"{name}.npz")
    w = hr.WORKLOADS[name]
    ctx = hr.Context(0)
    ctx.generate_synthetic(**w.synth())
    ctx.build_bvh()
    ctx.train_mlp(n_samples=400_000, steps=800, batch=4096, lr=2e-3, seed=1)
    arrs = scene_arrays_from_ctx(ctx)
    import sys
    sys.path.insert(0, str(GOLDEN))
    import make_golden

    same_scene = make_golden.digest(arrs) == str(z["digest"])
    print(f"{name}: scene digest {'equals' if same_scene else 'differs from'} the fixture's")
    yield name, w, z, ctx, ob.OracleScene(arrs)
    ctx.set_mode(hr.MODE_BATCHED)
    ctx.close()


def explain(g, ref, rays, order, count, osc, iso, trace):
    """Indices of the differing rays per explanation; 'unexplained' must be empty."""
    judge = osc.polish(rays, ref, iso)
    diff = np.where(~parity.same_hit(g, ref, judge))[0]
    out = {"differ": diff.size, "order_dependent": 0, "tie": 0, "grazing": 0, "second_root": 0, "unstable": 0,
           "unexplained": []}
    if diff.size == 0:
        return out
    replay = osc.trace_replay(rays[diff], iso, True, order[diff], count[diff], precision=32)
    ours, _ = osc.trace(rays[diff], iso, True, precision=32)
    od = parity.same_ids(replay, ref[diff]) & ~parity.same_ids(ours, ref[diff])
    out["order_dependent"] = int(od.sum())
    # order-dependent rays: the product against the oracle in its own order
    gi = np.where(od)[0]
    if gi.size:
        c = parity.classify(g[diff[gi]], ours[gi], rays[diff[gi]], osc, iso, product_trace=trace,
                            judge=osc.polish(rays[diff[gi]], ours[gi], iso))
        for k in ("tie", "grazing", "second_root", "unstable"):
            out[k] += c[k].size
        out["unexplained"] += list(diff[gi][c["other"]])
    # the rest: the product against the reference directly
    ri = np.where(~od)[0]
    if ri.size:
        c = parity.classify(g[diff[ri]], ref[diff[ri]], rays[diff[ri]], osc, iso, product_trace=trace,
                            judge=judge[diff[ri]])
        for k in ("tie", "grazing", "second_root", "unstable"):
            out[k] += c[k].size
        out["unexplained"] += list(diff[ri][c["other"]])
    return out


@pytest.mark.parametrize("mode", list(MODES))
def test_against_reference_and_judge(golden, mode):
    name, w, z, ctx, osc = golden
    ctx.set_mode(MODES[mode])
    rays = z["rays"]
    h = 1.0 / w.nx
    total = {}
    for iso in [float(v) for v in z["isovalues"]]:
        tag = iso_tag(iso)
        ref = ref_hits(z[f"trace_{tag}"])
        g = ctx.intersect(rays, iso, True)  # 0.0 traced as a real isovalue, as the fixture is
        st = ctx.stats()
        assert st["status"] == 0 and st["fp64_failed_after_fallback"] == 0
        # every ray the FP64 tie rule weighed carries the tie flag
        tied = (g["flags"] & hr.FLAG_TIE) != 0
        assert int(tied.sum()) == st["fp64_ties"] and st["fp64_ties_swapped"] <= st["fp64_ties"]
        # grazing hits (|cos| < 0.05 between ray and normal) are flagged and counted
        grazed = (g["flags"] & hr.FLAG_GRAZING) != 0
        assert int(grazed.sum()) == st["grazing_hits"]
        d = rays[:, 3:].astype(np.float64)
        cos = np.abs((g["n"].astype(np.float64) * d).sum(1)) / np.linalg.norm(d, axis=1)
        assert np.sum(grazed != ((g["kind"] > 0) & (cos < parity.GRAZE))) <= 2  # rounding at the bound

        def trace(r, iso=iso):
            return ctx.intersect(r, iso, True)

        ex = explain(g, ref, rays, z[f"order_{tag}"], z[f"count_{tag}"], osc, iso, trace)
        agree = 1.0 - ex["differ"] / rays.shape[0]
        print(f"{name} {mode} iso {iso}: rays {rays.shape[0]}, hits {int((ref['kind'] > 0).sum())}, identical "
              f"{agree:.4f}; differ {ex['differ']}: order-dependent {ex['order_dependent']}, tie {ex['tie']}, "
              f"grazing {ex['grazing']}, unstable {ex['unstable']}, unexplained {len(ex['unexplained'])}; "
              f"FP64 tie rule: weighed {st['fp64_ties']}, partner won {st['fp64_ties_swapped']}; "
              f"grazing hits {st['grazing_hits']}")
        for i in ex["unexplained"][:5]:
            print("   unexplained", i, g[i][["kind", "elem", "face", "t"]], ref[i][["kind", "elem", "face", "t"]])
        assert not ex["unexplained"]
        assert agree > 0.97
        # errors against the reference's hits polished to exact roots
        judge = osc.polish(rays, ref, iso)
        assert (judge["pad"][ref["kind"] > 0] == 1).mean() > 0.999
        err = parity.errors(g, judge, rays, h)
        print(f"   errors vs FP64 judge: {err}")
        for lab, e in err.items():
            if e["n"]:
                assert e["t_max_over_h"] <= POS_TOL, (lab, e)
                assert e["xi_max"] <= XI_TOL, (lab, e)
                assert e["u_max"] <= U_TOL, (lab, e)
        total[iso] = ex
    assert sum((z[f"trace_{iso_tag(float(v))}"][:, 0] == 2).sum() for v in z["isovalues"]) > 20


def test_hex4_against_reference():
    """The small scene's 4096 camera rays (iso 0.2 and faces only): every
    difference explained, t within the bound of the judge."""
    z = np.load(GOLDEN / "hex4_p4.npz")
    ctx, w = hr.workload_context("hex4_p4")
    osc = ob.OracleScene(scene_arrays_from_ctx(ctx))
    rays = z["rays"]
    for iso, on, key in ((float(z["isovalue"]), True, "iso"), (0.0, False, "faces")):
        ref = ref_hits(z[f"trace_{key}"])
        g = ctx.intersect(rays, iso, on)
        diff = np.where(~parity.same_ids(g, ref))[0]
        if diff.size:
            replay = osc.trace_replay(rays[diff], iso, on, z[f"order_{key}"][diff], z[f"count_{key}"][diff])
            ours, _ = osc.trace(rays[diff], iso, on, precision=32)
            od = parity.same_ids(replay, ref[diff]) & ~parity.same_ids(ours, ref[diff])
            rest = diff[~od]
            if rest.size:
                c = parity.classify(g[rest], ref[rest], rays[rest], osc, iso if on else 0.0,
                                    product_trace=lambda r: ctx.intersect(r, iso, on))
                assert c["other"].size == 0, c
        print(f"hex4 {key}: differ {diff.size}")
        judge = osc.polish(rays, ref, iso)
        for lab, e in parity.errors(g, judge, rays, 0.25).items():
            if e["n"]:
                assert e["t_max_over_h"] <= POS_TOL, (lab, e)
    ctx.close()
