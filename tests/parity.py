"""Comparison of product hits with the oracle (TEST INFRASTRUCTURE: used by
the tests and by bench.py's error_vs_fp64 block, always as the checker).

Identity (kind, element, face) of a product hit is compared with the oracle's
answer for the same ray; t, xi, u and the isosurface position are compared
with the judge: the FP64 oracle's hit polished to the exact root of its own
defining equations (oracle_bind.OracleScene.polish), so the yardstick does not
carry the reference's stopping tolerances (face residual 1e-4, |u - iso|
1e-5).

Rays whose identity differs are classified:
  tie        both answers are hits at the same t (within TIE_T), on different
             elements or faces: one surface point claimed twice (a face shared
             by two elements, an edge of two faces, an isosurface root in the
             overlap of two elements' padded boxes);
  grazing    |d . n| < GRAZE at either answer's hit;
  second_root  the same kind, element and face, at another root of the same
             equations within SECOND_ROOT_T in t: the ray meets the face (or
             the element's isosurface) twice, close together, and the seed or
             sample that converges first picks one; the product's hit is an
             exact root itself (the judge's polish started from it stays
             there);
  unstable   the reference algorithm's own answer is not stable on the ray:
             the FP32 and FP64 oracles disagree, or either changes its answer
             when the ray is turned by up to 4e-5 radians (NUDGE_ANGLES: a
             7th of a pixel at 3840 pixels over 60 degrees; 8 directions at
             each angle), or, where the caller passes the product's own
             tracer, the product's answer changes under the same turns. The
             ray then sits at a decision boundary of the algorithm: a sign
             change of u - iso at a scan sample, an inverse map that converges
             in one rounding and not in another (the reference skips such a
             sample, and a failed solve in the refinement turns the
             candidate's isosurface hit into a face test), the acceptance edge
             of a face, the clipping bound;
  other      none of these (a failure).
"""
from __future__ import annotations

import numpy as np

TIE_T = 1e-4      # the reference's face tolerance, in world units
GRAZE = 0.05      # |cos| of the angle between the ray and the surface normal
NUDGE_ANGLES = (2e-6, 1e-5, 4e-5)  # radians
N_NUDGE = 8 * len(NUDGE_ANGLES)
CLASSES = ("tie", "grazing", "second_root", "unstable", "other")
SECOND_ROOT_T = 1e-2  # world units: two roots of one face / one element's field this close


def ids(h) -> np.ndarray:
    return np.stack([np.asarray(h["kind"]).astype(np.int64), np.asarray(h["elem"]).astype(np.int64),
                     np.asarray(h["face"]).astype(np.int64)], 1)


def same_ids(a, b) -> np.ndarray:
    return np.all(ids(a) == ids(b), axis=1)


ROOT_T = 1e-3     # two hits of the same element and face further apart than this are different roots


def same_hit(gpu, ref, judge=None) -> np.ndarray:
    """Same kind, element and face and, for hits, the same root: within
    ROOT_T of the judge's t (the reference's own t where no judge is given)."""
    s = same_ids(gpu, ref)
    t_ref = np.asarray((judge if judge is not None else ref)["t"], np.float64)
    near = np.abs(np.asarray(gpu["t"], np.float64) - t_ref) <= ROOT_T
    return s & ((np.asarray(ref["kind"]) == 0) | near)


def nudged(rays: np.ndarray) -> np.ndarray:
    """Copies of each ray with the direction turned by NUDGE_ANGLES radians
    towards 8 fixed directions of the plane normal to it (the origin kept):
    N_NUDGE rays per ray, in ray-major order."""
    r = np.asarray(rays, np.float64).reshape(-1, 6)
    d = r[:, 3:] / np.linalg.norm(r[:, 3:], axis=1, keepdims=True)
    helper = np.where(np.abs(d[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    u = np.cross(d, helper)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    v = np.cross(d, u)
    out = np.zeros((r.shape[0], N_NUDGE, 6))
    out[:, :, :3] = r[:, None, :3]
    k = 0
    for ang in NUDGE_ANGLES:
        for j in range(8):
            a = np.pi * j / 4
            d2 = d + ang * (np.cos(a) * u + np.sin(a) * v)
            out[:, k, 3:] = d2 / np.linalg.norm(d2, axis=1, keepdims=True)
            k += 1
    return out.reshape(-1, 6).astype(np.float32)


def _varies(hits, base_ids, n) -> np.ndarray:
    return ~np.all(ids(hits).reshape(n, N_NUDGE, 3) == base_ids[:, None, :], axis=(1, 2))


def classify(gpu, ora, rays, osc, iso, product_trace=None, iso_on=True, judge=None) -> dict:
    """Classes of the identity differences between gpu (product hits) and ora
    (the oracle's or the reference's hits on the same rays at isovalue iso):
    a different kind, element or face, or the same ones at a different root
    (same_hit; judge: ora's hits polished, if available). product_trace(rays)
    -> product hits, optional: lets the product's own answer under the nudges
    count for 'unstable'. Returns the number of rays, of differing rays, and
    the indices of the differing rays per class."""
    diff = np.where(~same_hit(gpu, ora, judge))[0]
    out = {"rays": int(len(ora)), "differ": int(diff.size)}
    for k in CLASSES:
        out[k] = np.zeros(0, np.int64)
    if diff.size == 0:
        return out
    g, o, r = gpu[diff], ora[diff], np.asarray(rays)[diff]
    both = (g["kind"] > 0) & (o["kind"] > 0)
    tie = both & (np.abs(g["t"].astype(np.float64) - np.asarray(o["t"], np.float64)) <= TIE_T)
    d = r[:, 3:].astype(np.float64)
    gn = np.abs((np.asarray(g["n"], np.float64) * d).sum(1))
    on = np.abs((np.asarray(o["n"], np.float64) * d).sum(1))
    graz = ~tie & (((g["kind"] > 0) & (gn < GRAZE)) | ((o["kind"] > 0) & (on < GRAZE)))
    # same element and face at another root: the product's hit must be an
    # exact root of the same equations (the judge's polish leaves it there)
    second = np.zeros(diff.size, bool)
    cand = np.where(~tie & ~graz & both & same_ids(g, o) &
                    (np.abs(g["t"].astype(np.float64) - np.asarray(o["t"], np.float64)) <= SECOND_ROOT_T))[0]
    if cand.size:
        gp = osc.polish(r[cand], g[cand], iso)
        t0 = g["t"][cand].astype(np.float64)
        second[cand] = (gp["pad"] == 1) & (np.abs(gp["t"] - t0) <= 1e-6 * np.maximum(1.0, np.abs(t0)))
    rest = np.where(~tie & ~graz & ~second)[0]
    unstable = np.zeros(diff.size, bool)
    if rest.size:
        rr = r[rest]
        nr = nudged(rr)
        b32, _ = osc.trace(rr, iso, iso_on, precision=32)
        b64, _ = osc.trace(rr, iso, iso_on, precision=64)
        varies = ~same_hit(b32, b64)
        for prec, base in ((64, ids(b64)), (32, ids(b32))):
            hn, _ = osc.trace(nr, iso, iso_on, precision=prec)
            varies |= _varies(hn, base, rest.size)
        if product_trace is not None:
            varies |= _varies(product_trace(nr), ids(g[rest]), rest.size)
        unstable[rest] = varies
    other = ~tie & ~graz & ~second & ~unstable
    out["tie"], out["grazing"], out["second_root"] = diff[tie], diff[graz], diff[second]
    out["unstable"], out["other"] = diff[unstable], diff[other]
    return out


def counts(cls: dict) -> dict:
    return {k: (int(v.size) if isinstance(v, np.ndarray) else v) for k, v in cls.items()}


def root_off_face(hits) -> np.ndarray:
    """Face hits whose free reference coordinates lie beyond 1.05: the face
    equation's root is off the face (the reference accepts a face hit up to
    1.001 at a residual of 1e-4, so an accepted hit's exact root can lie
    outside). The product keeps such a hit as the solver returned it rather
    than move it off the face, so its error is stated against the solver's
    tolerance, not the root."""
    xi = np.abs(np.asarray(hits["xi"], np.float64))
    fixed = np.argmin(np.abs(xi - 1.0), axis=1)
    free = xi.copy()
    free[np.arange(xi.shape[0]), fixed] = 0.0
    return (np.asarray(hits["kind"]) == 1) & (free.max(1) > 1.05)


def errors(gpu, judge, rays, h: float) -> dict:
    """Errors of the product's hits against the judge on the rays whose
    identity agrees and whose judge polish converged (judge['pad'] == 1).
    t (= the position along the unit ray) in units of the element size h; xi
    and u absolute. Face hits whose root lies off the face (root_off_face)
    are counted apart."""
    ok = same_hit(gpu, judge, judge) & (judge["kind"] > 0) & (judge["pad"] == 1)
    off = ok & root_off_face(judge)
    ok &= ~off
    # grazing hits (|cos| < GRAZE): near a tangent the ray meets the surface
    # twice, close together, and either root may be the one polished
    d = np.asarray(rays, np.float64)[:, 3:]
    cos = np.abs((np.asarray(judge["n"], np.float64) * d).sum(1)) / np.maximum(np.linalg.norm(d, axis=1), 1e-30)
    graze = ok & (cos < GRAZE)
    ok &= ~graze
    off_t = float(np.abs(np.asarray(gpu["t"][off], np.float64) - judge["t"][off]).max()) if off.any() else 0.0
    res = {}
    for kind, lab in ((1, "face"), (2, "iso")):
        m = ok & (gpu["kind"] == kind)
        if not m.any():
            res[lab] = {"n": 0}
            if kind == 1:
                res[lab].update(root_off_face=int(off.sum()), root_off_face_t_max=off_t)
            continue
        dt = np.abs(gpu["t"][m].astype(np.float64) - judge["t"][m])
        # xi and u where both preimages lie in the padded element (|xi| <= 1.5):
        # beyond it the map need not be one to one, and the same point can
        # have another preimage (and field value) there
        gx, jx = np.asarray(gpu["xi"][m], np.float64), np.asarray(judge["xi"][m], np.float64)
        inside = (np.abs(gx).max(1) <= 1.5) & (np.abs(jx).max(1) <= 1.5)
        dxi = np.abs(gx - jx).max(1)[inside]
        du = np.abs(gpu["u"][m].astype(np.float64) - judge["u"][m])[inside]
        if not inside.any():
            dxi = du = np.zeros(1)
        # hits whose reference coordinates lie outside the element ([-1, 1]^3
        # by more than 1e-4): isosurface roots found in the padded box's
        # extrapolation beyond the element, as the reference finds them
        outside = int((np.abs(gx).max(1) > 1.0 + 1e-4).sum())
        res[lab] = {"n": int(m.sum()), "xi_outside_element": outside, "t_max_over_h": float(dt.max() / h),
                    "t_p99_over_h": float(np.quantile(dt, .99) / h), "xi_max": float(dxi.max()),
                    "xi_p99": float(np.quantile(dxi, .99)), "u_max": float(du.max()),
                    "u_p99": float(np.quantile(du, .99)), "other_preimage": int((~inside).sum())}
        res[lab]["grazing"] = int((graze & (gpu["kind"] == kind)).sum())
        if kind == 1:
            res[lab].update(root_off_face=int(off.sum()), root_off_face_t_max=off_t)
    return res


POS_TOL = 1e-5    # hit position error bound, in element sizes
XI_TOL = 5e-5     # reference coordinates (xi steps are world steps over |J|, about h / 2)
U_TOL = 1e-5


def check_against_oracle(gpu, rays, osc, iso, iso_on, h, product_trace=None, label=""):
    """The product's hits on given rays against the FP64 oracle: every
    identity difference classified (no 'other'), and t / xi / u of the
    agreeing hits within POS_TOL * h / XI_TOL / U_TOL of the judge (the
    oracle's hits polished to exact roots). Returns the class counts."""
    ref, _ = osc.trace(rays, iso, iso_on, precision=64)
    judge = osc.polish(rays, ref, iso)
    c = classify(gpu, ref, rays, osc, iso, product_trace=product_trace, iso_on=iso_on, judge=judge)
    cnt = counts(c)
    print(f"{label}: {cnt}")
    for i in c["other"][:5]:
        print("   other", i, gpu[i][["kind", "elem", "face", "t"]], ref[i][["kind", "elem", "face", "t"]])
    assert c["other"].size == 0, cnt
    err = errors(gpu, judge, rays, h)
    print(f"   errors vs FP64 judge: {err}")
    # a face hit kept as the solver returned it: within the face solver's tolerance
    assert err["face"]["root_off_face_t_max"] < 2e-3, err
    for lab, e in err.items():
        if e["n"]:
            assert e["t_max_over_h"] <= POS_TOL, (lab, e)
            assert e["xi_max"] <= XI_TOL, (lab, e)
            assert e["u_max"] <= U_TOL, (lab, e)
    return cnt
