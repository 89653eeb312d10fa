// CPU oracle for the non-hexahedral primitives: prisms, quads and curved
// triangles (TEST INFRASTRUCTURE ONLY, like horender_oracle.hpp; the GPU
// product never links or includes it).
//
// Restates, templated on the real type R, the reference's per-primitive
// algorithms: the modal maps (Modified-A x Modified-A x Modified-B for the
// prism, A x A for the quad, A x B for the triangle), the sampled boxes, and
// the three ray intersections with their start searches and Newton loops
// (FEM-AABB/fem/PrismElement.cu, QuadElement.cu, TriElement.cu). Operations
// are grouped the way those files group them, so that the FP32 instantiation
// built with -ffp-contract=off reproduces the reference's host build bit for
// bit; the FP64 instantiation runs the same steps in double.
#pragma once

#include "horender_oracle.hpp"

namespace horacle {

// base^power by repeated multiplication from 1 (ModalBasis.cuh:8-14)
template <class R> R ipow(R base, unsigned power) {
  R r = R(1);
  for (unsigned i = 0; i < power; ++i) r *= base;
  return r;
}

// Modified-B mode (i, j) at x and its derivative (ModalBasis.cuh:72-106)
template <class R> R mod_b(unsigned i, unsigned j, R x) {
  if (i == 0) return mod_a<R>(j, x);
  const R half_down = ipow<R>((R(1) - x) * R(0.5), i);
  if (j == 0) return half_down;
  R v = half_down;
  v *= R(0.5) * (R(1) + x);
  v *= jacobi<R>(static_cast<int>(j) - 1, R(2) * static_cast<R>(i) - R(1), R(1), x);
  return v;
}

template <class R> R mod_b_prime(unsigned i, unsigned j, R x) {
  if (i == 0) return mod_a_prime<R>(j, x);
  if (j == 0) {
    R v = -static_cast<R>(i);
    v *= ipow<R>(R(1) - x, i - 1);
    v *= ipow<R>(R(0.5), i);
    return v;
  }
  const R a = R(2) * static_cast<R>(i) - R(1);
  const R scale = ipow<R>(R(0.5), i + 1);
  const R p = jacobi<R>(static_cast<int>(j) - 1, a, R(1), x);
  const R dp = jacobi_deriv<R>(static_cast<int>(j) - 1, a, R(1), x);
  const R down_i = ipow<R>(R(1) - x, i);
  const R term1 = down_i * p;
  const R term2 = static_cast<R>(i) * ipow<R>(R(1) - x, i - 1) * (R(1) + x) * p;
  const R term3 = down_i * (R(1) + x) * dp;
  return scale * (term1 - term2 + term3);
}

enum PrimKind { PK_PRISM = 0, PK_QUAD = 1, PK_TRI = 2 };

// One primitive as the reference's Prism/Quad/TriElementData holds it:
// vertices (6 / 4 / 3), optional modal geometry (x, y, z blocks) and field.
// Modes: prism (mx, my, mz); quad and triangle (mx, my, -).
struct Prim {
  int kind;
  const float* geom[3];
  unsigned gm[3];
  const float* field;
  unsigned fm[3];
  float verts[6][3];
};

inline bool prim_has_geom(const Prim& p) {
  if (!p.geom[0] || !p.geom[1] || !p.geom[2] || p.gm[0] == 0 || p.gm[1] == 0) return false;
  return p.kind != PK_PRISM || p.gm[2] > 0;
}

// Number of coefficients of one component block.
inline int64_t prim_block_size(int kind, const unsigned m[3]) {
  if (kind == PK_QUAD) return int64_t(m[0]) * m[1];
  int64_t n = 0;
  const unsigned top = kind == PK_PRISM ? m[2] : m[1];
  for (unsigned i = 0; i < m[0]; ++i) n += top > i ? top - i : 0;
  return kind == PK_PRISM ? n * m[1] : n;
}

template <class R> V3<R> pvert(const Prim& p, int v) {
  return mk<R>(static_cast<R>(p.verts[v][0]), static_cast<R>(p.verts[v][1]), static_cast<R>(p.verts[v][2]));
}

// ---------------------------------------------------------------------------
// Modal sums. Which factor is differentiated: 0 none, 1 r, 2 s, 3 t.
// ---------------------------------------------------------------------------

// Prism: i (r) outermost, then j (s), then k < mz - i (t) (PrismElement.cu:15-103)
template <class R> R prism_modal(const float* c, const unsigned m[3], const V3<R>& x, int d) {
  if (!c || m[0] == 0 || m[1] == 0 || m[2] == 0) return R(0);
  R sum = R(0);
  int idx = 0;
  for (unsigned i = 0; i < m[0]; ++i) {
    const R ri = d == 1 ? mod_a_prime<R>(i, x.x) : mod_a<R>(i, x.x);
    for (unsigned j = 0; j < m[1]; ++j) {
      const R sj = d == 2 ? mod_a_prime<R>(j, x.y) : mod_a<R>(j, x.y);
      const unsigned top = m[2] > i ? m[2] - i : 0;
      for (unsigned k = 0; k < top; ++k) {
        const R tk = d == 3 ? mod_b_prime<R>(i, k, x.z) : mod_b<R>(i, k, x.z);
        sum += static_cast<R>(c[idx++]) * ri * sj * tk;
      }
    }
  }
  return sum;
}

// Quad: j (s) outer, i (r) inner (QuadElement.cu:22-74)
template <class R> R quad_modal(const float* c, const unsigned m[3], R r, R s, int d) {
  if (!c) return R(0);
  R sum = R(0);
  int idx = 0;
  for (unsigned j = 0; j < m[1]; ++j) {
    const R sj = d == 2 ? mod_a_prime<R>(j, s) : mod_a<R>(j, s);
    for (unsigned i = 0; i < m[0]; ++i) {
      const R ri = d == 1 ? mod_a_prime<R>(i, r) : mod_a<R>(i, r);
      sum += static_cast<R>(c[idx++]) * ri * sj;
    }
  }
  return sum;
}

// Triangle: i (r, Modified-A) outer, j < my - i (s, Modified-B) inner (TriElement.cu:46-100)
template <class R> R tri_modal(const float* c, const unsigned m[3], R r, R s, int d) {
  if (!c || m[0] == 0 || m[1] == 0) return R(0);
  R sum = R(0);
  int idx = 0;
  for (unsigned i = 0; i < m[0]; ++i) {
    const R ai = d == 1 ? mod_a_prime<R>(i, r) : mod_a<R>(i, r);
    const unsigned top = m[1] > i ? m[1] - i : 0;
    for (unsigned j = 0; j < top; ++j) {
      const R bj = d == 2 ? mod_b_prime<R>(i, j, s) : mod_b<R>(i, j, s);
      sum += static_cast<R>(c[idx++]) * ai * bj;
    }
  }
  return sum;
}

// ---------------------------------------------------------------------------
// Maps and Jacobians
// ---------------------------------------------------------------------------

// Linear prism (PrismElement.cu:186-216): bottom quad 0-3 weighted
// (1 -/+ r)(1 -/+ s)(1 - t)/8, top edge 4-5 weighted (1 -/+ s)(1 + t)/4.
template <class R> V3<R> prism_map(const Prim& p, const V3<R>& x) {
  if (prim_has_geom(p))
    return mk<R>(prism_modal<R>(p.geom[0], p.gm, x, 0), prism_modal<R>(p.geom[1], p.gm, x, 0),
                 prism_modal<R>(p.geom[2], p.gm, x, 0));
  const R r = x.x, s = x.y, t = x.z;
  const R w[6] = {R(0.125) * ((R(1) - r) * (R(1) - s) * (R(1) - t)), R(0.125) * ((R(1) + r) * (R(1) - s) * (R(1) - t)),
                  R(0.125) * ((R(1) + r) * (R(1) + s) * (R(1) - t)), R(0.125) * ((R(1) - r) * (R(1) + s) * (R(1) - t)),
                  R(0.25) * ((R(1) - s) * (R(1) + t)), R(0.25) * ((R(1) + s) * (R(1) + t))};
  V3<R> out = mk<R>(0, 0, 0);
  for (int v = 0; v < 6; ++v) {
    const V3<R> pv = pvert<R>(p, v);
    out.x += w[v] * pv.x;
    out.y += w[v] * pv.y;
    out.z += w[v] * pv.z;
  }
  return out;
}

// J[3*component + (r, s, t)]. The linear form is the reference's
// (PrismElement.cu:228-279), including its extra 0.5 (1 + r) dr term in dt.
template <class R> void prism_jac(const Prim& p, const V3<R>& x, R J[9]) {
  if (prim_has_geom(p)) {
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) J[3 * a + d] = prism_modal<R>(p.geom[a], p.gm, x, d + 1);
    return;
  }
  const R rm = R(1) - x.x, rp = R(1) + x.x, sm = R(1) - x.y, sp = R(1) + x.y, tm = R(1) - x.z, tp = R(1) + x.z;
  for (int a = 0; a < 3; ++a) {
    const R v0 = p.verts[0][a], v1 = p.verts[1][a], v2 = p.verts[2][a], v3 = p.verts[3][a], v4 = p.verts[4][a],
            v5 = p.verts[5][a];
    const R dr = R(0.25) * (-sm * v0 + sm * v1 + sp * v2 - sp * v3);
    const R ds = R(0.125) * (-rm * v0 - rp * v1 + rp * v2 + rm * v3) * tm + R(0.25) * (-tp * v4 + tp * v5);
    const R dt = R(0.125) * (-rm * sm * v0 - rp * sm * v1 - rp * sp * v2 - rm * sp * v3) +
                 R(0.25) * (sm * v4 + sp * v5) + R(0.5) * rp * dr;
    J[3 * a + 0] = dr;
    J[3 * a + 1] = ds;
    J[3 * a + 2] = dt;
  }
}

// Bilinear quad with vertex v at r = (v & 1 ? 1 : -1), s = (v & 2 ? 1 : -1)
// (QuadElement.cu:15-20, 106-118)
template <class R> V3<R> quad_map(const Prim& p, R r, R s) {
  if (prim_has_geom(p))
    return mk<R>(quad_modal<R>(p.geom[0], p.gm, r, s, 0), quad_modal<R>(p.geom[1], p.gm, r, s, 0),
                 quad_modal<R>(p.geom[2], p.gm, r, s, 0));
  V3<R> out = mk<R>(0, 0, 0);
  for (int v = 0; v < 4; ++v) {
    const R rs = (v & 1) ? R(1) : R(-1), ss = (v & 2) ? R(1) : R(-1);
    const R w = R(0.25) * (R(1) + rs * r) * (R(1) + ss * s);
    const V3<R> pv = pvert<R>(p, v);
    out.x += w * pv.x;
    out.y += w * pv.y;
    out.z += w * pv.z;
  }
  return out;
}

template <class R> void quad_jac(const Prim& p, R r, R s, V3<R>& dr, V3<R>& ds) {
  if (prim_has_geom(p)) {
    dr = mk<R>(quad_modal<R>(p.geom[0], p.gm, r, s, 1), quad_modal<R>(p.geom[1], p.gm, r, s, 1),
               quad_modal<R>(p.geom[2], p.gm, r, s, 1));
    ds = mk<R>(quad_modal<R>(p.geom[0], p.gm, r, s, 2), quad_modal<R>(p.geom[1], p.gm, r, s, 2),
               quad_modal<R>(p.geom[2], p.gm, r, s, 2));
    return;
  }
  dr = mk<R>(0, 0, 0);
  ds = mk<R>(0, 0, 0);
  for (int v = 0; v < 4; ++v) {
    const R rs = (v & 1) ? R(1) : R(-1), ss = (v & 2) ? R(1) : R(-1);
    const R wr = R(0.25) * rs * (R(1) + ss * s);
    const R ws = R(0.25) * ss * (R(1) + rs * r);
    const V3<R> pv = pvert<R>(p, v);
    dr.x += wr * pv.x;
    dr.y += wr * pv.y;
    dr.z += wr * pv.z;
    ds.x += ws * pv.x;
    ds.y += ws * pv.y;
    ds.z += ws * pv.z;
  }
}

// Reference (r, s) -> clamped barycentric (u, v) (TriElement.cu:17-31)
template <class R> void tri_bary(R r, R s, R& u, R& v) {
  u = R(0.5) * (r + R(1));
  v = R(0.5) * (s + R(1));
  u = rmin<R>(rmax<R>(u, R(0)), R(1));
  v = rmin<R>(rmax<R>(v, R(0)), R(1));
  if (u + v > R(1)) {
    const R excess = u + v - R(1);
    u -= R(0.5) * excess;
    v -= R(0.5) * excess;
    u = rmax<R>(u, R(0));
    v = rmax<R>(v, R(0));
  }
}

template <class R> V3<R> tri_map(const Prim& p, R r, R s) {
  if (prim_has_geom(p))
    return mk<R>(tri_modal<R>(p.geom[0], p.gm, r, s, 0), tri_modal<R>(p.geom[1], p.gm, r, s, 0),
                 tri_modal<R>(p.geom[2], p.gm, r, s, 0));
  R u, v;
  tri_bary<R>(r, s, u, v);
  const R w = rmax<R>(R(0), R(1) - u - v);
  const V3<R> a = pvert<R>(p, 0), b = pvert<R>(p, 1), c = pvert<R>(p, 2);
  V3<R> out = mk<R>(0, 0, 0);
  out.x += w * a.x; out.y += w * a.y; out.z += w * a.z;
  out.x += u * b.x; out.y += u * b.y; out.z += u * b.z;
  out.x += v * c.x; out.y += v * c.y; out.z += v * c.z;
  return out;
}

template <class R> void tri_jac(const Prim& p, R r, R s, V3<R>& dr, V3<R>& ds) {
  if (prim_has_geom(p)) {
    dr = mk<R>(tri_modal<R>(p.geom[0], p.gm, r, s, 1), tri_modal<R>(p.geom[1], p.gm, r, s, 1),
               tri_modal<R>(p.geom[2], p.gm, r, s, 1));
    ds = mk<R>(tri_modal<R>(p.geom[0], p.gm, r, s, 2), tri_modal<R>(p.geom[1], p.gm, r, s, 2),
               tri_modal<R>(p.geom[2], p.gm, r, s, 2));
    return;
  }
  const V3<R> a = pvert<R>(p, 0), b = pvert<R>(p, 1), c = pvert<R>(p, 2);
  dr = mk<R>(R(0.5) * (b.x - a.x), R(0.5) * (b.y - a.y), R(0.5) * (b.z - a.z));
  ds = mk<R>(R(0.5) * (c.x - a.x), R(0.5) * (c.y - a.y), R(0.5) * (c.z - a.z));
}

// Surface or volume point of a primitive at reference coordinates x (the
// surfaces use x.x, x.y).
template <class R> V3<R> prim_map(const Prim& p, const V3<R>& x) {
  if (p.kind == PK_PRISM) return prism_map<R>(p, x);
  if (p.kind == PK_QUAD) return quad_map<R>(p, x.x, x.y);
  return tri_map<R>(p, x.x, x.y);
}

// Field value at x (EvaluatePrismField / EvaluateQuadField / EvaluateTriangleField).
template <class R> R prim_field(const Prim& p, const V3<R>& x) {
  if (p.kind == PK_PRISM) return prism_modal<R>(p.field, p.fm, x, 0);
  if (p.kind == PK_QUAD) return quad_modal<R>(p.field, p.fm, x.x, x.y, 0);
  return tri_modal<R>(p.field, p.fm, x.x, x.y, 0);
}

// ---------------------------------------------------------------------------
// Sampled boxes (ComputePrismAabb 4 per axis, ComputeQuadAabb 4 per axis,
// ComputeTriangleAabb 6 per edge, high-order geometry only)
// ---------------------------------------------------------------------------
template <class R> void prim_box(const Prim& p, R lo[3], R hi[3]) {
  for (int a = 0; a < 3; ++a) {
    lo[a] = static_cast<R>(FLT_MAX);
    hi[a] = static_cast<R>(-FLT_MAX);
  }
  auto grow = [&](const V3<R>& q) {
    lo[0] = rmin<R>(lo[0], q.x); lo[1] = rmin<R>(lo[1], q.y); lo[2] = rmin<R>(lo[2], q.z);
    hi[0] = rmax<R>(hi[0], q.x); hi[1] = rmax<R>(hi[1], q.y); hi[2] = rmax<R>(hi[2], q.z);
  };
  const int nv = p.kind == PK_PRISM ? 6 : (p.kind == PK_QUAD ? 4 : 3);
  for (int v = 0; v < nv; ++v) grow(pvert<R>(p, v));
  if (p.kind == PK_TRI) {
    if (!prim_has_geom(p)) return;
    const int n = 6;
    for (int i = 0; i <= n; ++i)
      for (int j = 0; j <= n - i; ++j) {
        const R u = static_cast<R>(i) / static_cast<R>(n), v = static_cast<R>(j) / static_cast<R>(n);
        grow(tri_map<R>(p, R(2) * u - R(1), R(2) * v - R(1)));
      }
    return;
  }
  const int n = 4;
  auto at = [&](int i) { return R(-1) + R(2) * static_cast<R>(i) / static_cast<R>(n - 1); };
  if (p.kind == PK_QUAD) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) grow(quad_map<R>(p, at(i), at(j)));
    return;
  }
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) grow(prism_map<R>(p, mk<R>(at(i), at(j), at(k))));
}

// ---------------------------------------------------------------------------
// Small helpers shared by the three intersections
// ---------------------------------------------------------------------------

// Ray parameter of the point of the ray closest to q.
template <class R> R ray_param(const Ray<R>& ray, const V3<R>& q) {
  const V3<R> d = mk<R>(q.x - ray.o.x, q.y - ray.o.y, q.z - ray.o.z);
  const R dd = dot3<R>(ray.d, ray.d);
  return dd > R(0) ? dot3<R>(d, ray.d) / dd : R(0);
}

template <class R> V3<R> ray_at(const Ray<R>& ray, R t) {
  return mk<R>(ray.o.x + t * ray.d.x, ray.o.y + t * ray.d.y, ray.o.z + t * ray.d.z);
}

// x = A^-1 b through the adjugate; false when |det| < 1e-12 (Solve3x3).
template <class R> bool solve3(const R A[9], const V3<R>& b, V3<R>& x) {
  const R det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                A[2] * (A[3] * A[7] - A[4] * A[6]);
  if (rabs<R>(det) < static_cast<R>(1e-12f)) return false;
  const R id = R(1) / det;
  R v[9];
  v[0] = (A[4] * A[8] - A[5] * A[7]) * id;
  v[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  v[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  v[3] = (A[5] * A[6] - A[3] * A[8]) * id;
  v[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  v[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  v[6] = (A[3] * A[7] - A[4] * A[6]) * id;
  v[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  v[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  x = mk<R>(v[0] * b.x + v[1] * b.y + v[2] * b.z, v[3] * b.x + v[4] * b.y + v[5] * b.z,
            v[6] * b.x + v[7] * b.y + v[8] * b.z);
  return true;
}

template <class R> R max_abs3(const V3<R>& v) { return rmax<R>(rabs<R>(v.x), rmax<R>(rabs<R>(v.y), rabs<R>(v.z))); }

// Gauss-Newton projection of a point onto a surface primitive from a start
// (SolveWithInitialGuess of QuadElement.cu:178-211 / TriElement.cu:186-222).
template <class R> bool surf_project(const Prim& p, const V3<R>& q, R r0, R s0, R& r, R& s, int iters, R tol) {
  r = r0;
  s = s0;
  for (int it = 0; it < iters; ++it) {
    const V3<R> m = p.kind == PK_QUAD ? quad_map<R>(p, r, s) : tri_map<R>(p, r, s);
    const V3<R> diff = mk<R>(m.x - q.x, m.y - q.y, m.z - q.z);
    V3<R> dr, ds;
    if (p.kind == PK_QUAD) quad_jac<R>(p, r, s, dr, ds);
    else tri_jac<R>(p, r, s, dr, ds);
    const R g00 = dot3<R>(dr, dr), g01 = dot3<R>(dr, ds), g11 = dot3<R>(ds, ds);
    const R det = g00 * g11 - g01 * g01;
    if (rabs<R>(det) < static_cast<R>(1e-10f)) return false;
    const R id = R(1) / det;
    const R b0 = dot3<R>(dr, diff), b1 = dot3<R>(ds, diff);
    const R dR = id * (g11 * b0 - g01 * b1);
    const R dS = id * (-g01 * b0 + g00 * b1);
    r -= dR;
    s -= dS;
    if (rabs<R>(dR) < tol && rabs<R>(dS) < tol) return true;
  }
  return false;
}

// QuadContainsPoint (QuadElement.cu:224-250): 9 starts, Newton tolerance
// 1e-4, accepted inside [-1.05, 1.05]^2 when it maps back within 5e-4.
template <class R> bool quad_contains(const Prim& p, const V3<R>& q, R& r_out, R& s_out) {
  static const float seeds[9][2] = {{0.f, 0.f},  {-0.5f, -0.5f}, {0.5f, -0.5f}, {-0.5f, 0.5f}, {0.5f, 0.5f},
                                    {-0.9f, -0.9f}, {0.9f, -0.9f}, {-0.9f, 0.9f}, {0.9f, 0.9f}};
  const R lim = static_cast<R>(1.05f), back = static_cast<R>(5e-4f);
  for (const auto& sd : seeds) {
    R r, s;
    if (!surf_project<R>(p, q, sd[0], sd[1], r, s, 40, static_cast<R>(1e-4f))) continue;
    if (r < -lim || r > lim || s < -lim || s > lim) continue;
    const V3<R> m = quad_map<R>(p, r, s);
    if (rabs<R>(m.x - q.x) > back || rabs<R>(m.y - q.y) > back || rabs<R>(m.z - q.z) > back) continue;
    r_out = r;
    s_out = s;
    return true;
  }
  return false;
}

// TriangleContainsPoint (TriElement.cu:391-409): 4 starts of 30 iterations
// at tolerance 1e-4, then an inside test on the clamped barycentrics.
template <class R> bool tri_contains(const Prim& p, const V3<R>& q, R& r_out, R& s_out) {
  static const float seeds[4][2] = {{0.f, 0.f}, {-0.5f, -0.5f}, {0.5f, -0.5f}, {0.f, 0.5f}};
  R r = 0, s = 0;
  bool ok = false;
  for (const auto& sd : seeds)
    if (surf_project<R>(p, q, sd[0], sd[1], r, s, 30, static_cast<R>(1e-4f))) {
      ok = true;
      break;
    }
  if (!ok) return false;
  R u, v;
  tri_bary<R>(r, s, u, v);
  const R w = R(1) - u - v;
  const R e = static_cast<R>(-1e-3f);
  const bool inside = u >= e && v >= e && w >= e;
  if (inside) {
    r_out = r;
    s_out = s;
  }
  return inside;
}

// ---------------------------------------------------------------------------
// Ray intersections. On success t and the reference coordinates (r, s[, t]).
// ---------------------------------------------------------------------------

// IntersectRayWithPrism (PrismElement.cu:456-532): from each of 7 starts,
// move rst so that x(rst) meets the ray at the point closest to x(rst);
// accept when within 1e-5 and inside [-1.05, 1.05]^3. At most 60 steps a start.
template <class R> bool prism_intersect(const Prim& p, const R lo[3], const R hi[3], const Ray<R>& ray, R tmin, R tmax,
                                        R& t_hit, V3<R>& x_hit) {
  R enter, exit;
  if (!ray_box<R>(ray, mk<R>(lo[0], lo[1], lo[2]), mk<R>(hi[0], hi[1], hi[2]), tmin, tmax, enter, exit)) return false;
  static const float seeds[7][3] = {{0.f, 0.f, 0.f},     {-0.5f, -0.5f, -0.5f}, {0.5f, -0.5f, -0.5f}, {0.f, 0.5f, -0.5f},
                                    {-0.5f, 0.f, 0.5f}, {0.5f, 0.f, 0.5f},     {0.f, 0.5f, 0.5f}};
  const R tol = static_cast<R>(1e-5f), lim = static_cast<R>(1.05f);
  for (const auto& sd : seeds) {
    V3<R> x = mk<R>(sd[0], sd[1], sd[2]);
    for (int it = 0; it < 60; ++it) {
      const V3<R> m = prism_map<R>(p, x);
      const R tau = ray_param<R>(ray, m);
      if (tau < enter || tau > exit) break;
      const V3<R> q = ray_at<R>(ray, tau);
      const V3<R> res = mk<R>(m.x - q.x, m.y - q.y, m.z - q.z);
      if (max_abs3<R>(res) < tol && x.x >= -lim && x.x <= lim && x.y >= -lim && x.y <= lim && x.z >= -lim &&
          x.z <= lim) {
        t_hit = tau;
        x_hit = x;
        return true;
      }
      R J[9];
      prism_jac<R>(p, x, J);
      V3<R> dx;
      if (!solve3<R>(J, res, dx)) break;
      x.x -= dx.x;
      x.y -= dx.y;
      x.z -= dx.z;
    }
  }
  return false;
}

// Start of a surface intersection (InitializeQuadIntersection,
// QuadElement.cu:402-467; InitializeTriangleIntersection, TriElement.cu:224-291):
// the first of n_samples + 1 evenly spaced box-segment points that projects
// onto the surface, else the plane of vertices 0, 1 and 3 (quad) / 0, 1, 2
// (triangle) hit within the segment, else the segment's middle.
template <class R> bool surf_start(const Prim& p, const R lo[3], const R hi[3], const Ray<R>& ray, R tmin, R tmax,
                                   R& t0, R& r0, R& s0) {
  R enter, exit;
  if (!ray_box<R>(ray, mk<R>(lo[0], lo[1], lo[2]), mk<R>(hi[0], hi[1], hi[2]), tmin, tmax, enter, exit)) return false;
  const bool quad = p.kind == PK_QUAD;
  const int n = quad ? 10 : 8;
  auto contains = [&](const V3<R>& q, R& r, R& s) {
    return quad ? quad_contains<R>(p, q, r, s) : tri_contains<R>(p, q, r, s);
  };
  auto map = [&](R r, R s) { return quad ? quad_map<R>(p, r, s) : tri_map<R>(p, r, s); };
  for (int i = 0; i <= n; ++i) {
    const R u = static_cast<R>(i) / static_cast<R>(n);
    const R t = enter + (exit - enter) * u;
    R r, s;
    if (contains(ray_at<R>(ray, t), r, s)) {
      t0 = ray_param<R>(ray, map(r, s));
      r0 = r;
      s0 = s;
      return true;
    }
  }
  const V3<R> a = pvert<R>(p, 0), b = pvert<R>(p, 1), c = pvert<R>(p, quad ? 3 : 2);
  V3<R> nrm = cross3<R>(mk<R>(b.x - a.x, b.y - a.y, b.z - a.z), mk<R>(c.x - a.x, c.y - a.y, c.z - a.z));
  const R inv = R(1) / std::sqrt(dot3<R>(nrm, nrm));
  nrm = mk<R>(nrm.x * inv, nrm.y * inv, nrm.z * inv);
  const R den = dot3<R>(nrm, ray.d);
  const R mid = R(0.5) * (enter + exit);
  const R big = static_cast<R>(1e-6f);
  if (quad) {
    if (rabs<R>(den) > big) {
      R t = dot3<R>(nrm, mk<R>(a.x - ray.o.x, a.y - ray.o.y, a.z - ray.o.z)) / den;
      if (t < enter || t > exit) t = mid;
      R r, s;
      if (contains(ray_at<R>(ray, t), r, s)) {
        r0 = r;
        s0 = s;
        t0 = ray_param<R>(ray, map(r, s));
        return true;
      }
    }
    r0 = 0;
    s0 = 0;
    t0 = mid;
    return true;
  }
  R t = mid;
  if (rabs<R>(den) > big) {
    const R pt = dot3<R>(nrm, mk<R>(a.x - ray.o.x, a.y - ray.o.y, a.z - ray.o.z)) / den;
    if (pt >= enter && pt <= exit) t = pt;
  }
  R r, s;
  if (contains(ray_at<R>(ray, t), r, s)) {
    r0 = r;
    s0 = s;
  } else {
    r0 = 0;
    s0 = 0;
  }
  t0 = ray_param<R>(ray, map(r0, s0));
  return true;
}

// IntersectRayWithQuad (QuadElement.cu:469-527) / IntersectRayWithTriangle
// (TriElement.cu:451-497): Newton on (r, s, t) for x(r, s) = o + t d, at most
// 40 steps, tolerance 1e-5. The quad also wants (r, s) inside
// [-1.02, 1.02]^2 and stops when t leaves [tmin, tmax].
template <class R> bool surf_intersect(const Prim& p, const R lo[3], const R hi[3], const Ray<R>& ray, R tmin, R tmax,
                                       R& t_hit, V3<R>& x_hit) {
  R t, r, s;
  if (!surf_start<R>(p, lo, hi, ray, tmin, tmax, t, r, s)) return false;
  const bool quad = p.kind == PK_QUAD;
  const R tol = static_cast<R>(1e-5f), lim = static_cast<R>(1.02f);
  for (int it = 0; it < 40; ++it) {
    const V3<R> m = quad ? quad_map<R>(p, r, s) : tri_map<R>(p, r, s);
    const V3<R> q = ray_at<R>(ray, t);
    const V3<R> res = mk<R>(q.x - m.x, q.y - m.y, q.z - m.z);
    const bool close = max_abs3<R>(res) < tol;
    const bool inside = !quad || (r >= -lim && r <= lim && s >= -lim && s <= lim);
    if (close && inside && t >= tmin && t <= tmax) {
      t_hit = t;
      x_hit = mk<R>(r, s, R(0));
      return true;
    }
    V3<R> dr, ds;
    if (quad) quad_jac<R>(p, r, s, dr, ds);
    else tri_jac<R>(p, r, s, dr, ds);
    const R A[9] = {-dr.x, -ds.x, ray.d.x, -dr.y, -ds.y, ray.d.y, -dr.z, -ds.z, ray.d.z};
    V3<R> dx;
    if (!solve3<R>(A, mk<R>(-res.x, -res.y, -res.z), dx)) return false;
    r += dx.x;
    s += dx.y;
    t += dx.z;
    if (quad && (t < tmin || t > tmax)) return false;
  }
  return false;
}

template <class R> bool prim_intersect(const Prim& p, const R lo[3], const R hi[3], const Ray<R>& ray, R tmin, R tmax,
                                       R& t_hit, V3<R>& x_hit) {
  if (p.kind == PK_PRISM) return prism_intersect<R>(p, lo, hi, ray, tmin, tmax, t_hit, x_hit);
  return surf_intersect<R>(p, lo, hi, ray, tmin, tmax, t_hit, x_hit);
}

// Normal at a hit as raytracer.cu:283-289 / 309-314 / 334-339 forms it: the
// cross product of the r and s tangents, normalised, turned against the
// ray, then HitRecord::set_face_normal (geometry.h:87-90), which negates it
// once more when it is not strictly against the ray.
template <class R> V3<R> prim_normal(const Prim& p, const V3<R>& x, const V3<R>& d) {
  V3<R> a, b;
  if (p.kind == PK_PRISM) {
    R J[9];
    prism_jac<R>(p, x, J);
    a = mk<R>(J[0], J[3], J[6]);
    b = mk<R>(J[1], J[4], J[7]);
  } else if (p.kind == PK_QUAD) {
    quad_jac<R>(p, x.x, x.y, a, b);
  } else {
    tri_jac<R>(p, x.x, x.y, a, b);
  }
  V3<R> n = cross3<R>(a, b);
  const R inv = R(1) / std::sqrt(dot3<R>(n, n));
  n = mk<R>(n.x * inv, n.y * inv, n.z * inv);
  if (dot3<R>(n, d) > R(0)) n = mk<R>(-n.x, -n.y, -n.z);
  if (!(dot3<R>(d, n) < R(0))) n = mk<R>(-n.x, -n.y, -n.z);
  return n;
}

}  // namespace horacle
