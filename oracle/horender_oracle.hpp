// CPU oracle for the curved-hex ray / isosurface hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: the GPU product never
// links it, includes it or calls it. Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline arm may load the library built from it.
//
// It restates, in templated form (Real = float or double), the reference's
// per-element algorithm so that the same steps can be run in FP32 (to pin the
// restatement bit-for-bit against the reference's own host build) and in FP64
// (the judge of error for the GPU kernels). Each function names the reference
// file:line whose steps it follows. Reference paths are relative to the
// reference project's root (FEM-AABB/...).
//
// Candidate ordering: the reference visits candidate elements in BVH stack
// order (FEM-AABB/raytracer.cu:117-356), so its answer depends on the tree it
// happened to build. The oracle (and the GPU path) visit candidates in
// ascending (padded-box entry t, element index) order instead, with the same
// per-candidate policy and the same clipping of each candidate's segment to
// the closest hit so far. Both orders give the same hit except in rare cases
// where two candidates' results interact through that clipping; the parity
// harness counts those cases against the reference's own traversal order.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace horacle {

template <class R> struct V3 {
  R x, y, z;
};
template <class R> inline V3<R> mk(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline R comp(const V3<R>& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
template <class R> inline void setc(V3<R>& v, int a, R s) {
  if (a == 0) v.x = s; else if (a == 1) v.y = s; else v.z = s;
}
template <class R> inline R dot3(const V3<R>& a, const V3<R>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross3(const V3<R>& a, const V3<R>& b) {
  return mk<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> inline R rabs(R v) { return v < R(0) ? -v : v; }
template <class R> inline R rmin(R a, R b) { return std::fmin(a, b); }
template <class R> inline R rmax(R a, R b) { return std::fmax(a, b); }

// ---------------------------------------------------------------------------
// 1-D modal basis (FEM-AABB/fem/ModalBasis.cuh:16-70)
// ---------------------------------------------------------------------------

// Jacobi polynomial P_n^{(a,b)}(x) by the standard three-term recurrence,
// grouped the way ModalBasis.cuh:16-41 groups it so FP32 rounding agrees.
template <class R> R jacobi(int n, R a, R b, R x) {
  if (n == 0) return R(1);
  const R first = R(0.5) * ((R(2) + a + b) * x + (a - b));
  if (n == 1) return first;
  R older = R(1), newer = first, cur = R(0);
  for (int k = 2; k <= n; ++k) {
    const R kr = static_cast<R>(k);
    const R s = R(2) * kr + a + b;
    const R den = R(2) * kr * (kr + a + b) * (s - R(2));
    const R up = (s - R(1)) * (s * (s - R(2)) * x + (a * a - b * b)) * newer;
    const R down = R(2) * (kr + a - R(1)) * (kr + b - R(1)) * s * older;
    cur = (up - down) / den;
    older = newer;
    newer = cur;
  }
  return cur;
}

// d/dx P_n^{(a,b)} = (n+a+b+1)/2 * P_{n-1}^{(a+1,b+1)}  (ModalBasis.cuh:43-51)
template <class R> R jacobi_deriv(int n, R a, R b, R x) {
  if (n == 0) return R(0);
  const R f = R(0.5) * (static_cast<R>(n) + a + b + R(1));
  return f * jacobi(n - 1, a + R(1), b + R(1), x);
}

// Modified-A (Nektar "Modified_A") mode i at x  (ModalBasis.cuh:53-60)
template <class R> R mod_a(unsigned i, R x) {
  if (i == 0) return R(0.5) * (R(1) - x);
  if (i == 1) return R(0.5) * (R(1) + x);
  const R p = jacobi(static_cast<int>(i - 2), R(1), R(1), x);
  return R(0.25) * (R(1) - x * x) * p;
}

// derivative of mode i  (ModalBasis.cuh:62-70)
template <class R> R mod_a_prime(unsigned i, R x) {
  if (i == 0) return R(-0.5);
  if (i == 1) return R(0.5);
  const int m = static_cast<int>(i - 2);
  const R p = jacobi(m, R(1), R(1), x);
  const R dp = jacobi_deriv(m, R(1), R(1), x);
  return R(-0.5) * x * p + R(0.25) * (R(1) - x * x) * dp;
}

// ---------------------------------------------------------------------------
// Element view. Coefficients are always stored as float (the loader and the
// scene keep fp32, FEM-AABB/xml_fld_field_parser.cpp:151); arithmetic is R.
// Layout per element: modes (nx,ny,nz), coefficient index ((k*ny)+j)*nx+i
// (FEM-AABB/fem/HexElement.cu:14-26); geometry x block, then y, then z
// (FEM-AABB/raytracer.h:151-153).
// ---------------------------------------------------------------------------
struct Elem {
  const float* geom[3];   // nullptr => trilinear map from vertices
  unsigned gm[3];         // geometry modes
  const float* field;     // nullptr => no field
  unsigned fm[3];         // field modes
  float verts[8][3];      // corner vertices, XML order
};

inline bool has_ho_geom(const Elem& e) {
  return e.geom[0] && e.geom[1] && e.geom[2] && e.gm[0] > 0 && e.gm[1] > 0 && e.gm[2] > 0;
}

enum Deriv { D_NONE = 0, D_R = 1, D_S = 2, D_T = 3 };

// Triple-loop modal sum with one factor differentiated (HexElement.cu:8-94).
// The reference calls ModifiedA inside the innermost loop; the 1-D values
// only depend on (mode, coordinate), so they are computed once per call here
// — the same values, accumulated in the same order.
template <class R> R modal3(const float* c, const unsigned m[3], const V3<R>& p, Deriv d) {
  if (!c || m[0] == 0 || m[1] == 0 || m[2] == 0) return R(0);
  R br[16], bs[16], bt[16];
  for (unsigned i = 0; i < m[0]; ++i) br[i] = (d == D_R) ? mod_a_prime<R>(i, p.x) : mod_a<R>(i, p.x);
  for (unsigned j = 0; j < m[1]; ++j) bs[j] = (d == D_S) ? mod_a_prime<R>(j, p.y) : mod_a<R>(j, p.y);
  for (unsigned k = 0; k < m[2]; ++k) bt[k] = (d == D_T) ? mod_a_prime<R>(k, p.z) : mod_a<R>(k, p.z);
  R acc = R(0);
  int idx = 0;
  for (unsigned k = 0; k < m[2]; ++k)
    for (unsigned j = 0; j < m[1]; ++j)
      for (unsigned i = 0; i < m[0]; ++i) acc += static_cast<R>(c[idx++]) * br[i] * bs[j] * bt[k];
  return acc;
}

// XML vertex i sits at Z-order corner kXmlToZ[i] (HexElement.cu:104-120).
static const int kXmlToZ[8] = {0, 1, 3, 2, 4, 5, 7, 6};

template <class R> V3<R> map_trilinear(const Elem& e, const V3<R>& p) {
  V3<R> out = mk<R>(0, 0, 0);
  for (int v = 0; v < 8; ++v) {
    const int z = kXmlToZ[v];
    const R sr = (z & 1) ? R(1) : R(-1), ss = (z & 2) ? R(1) : R(-1), st = (z & 4) ? R(1) : R(-1);
    const R w = R(0.125) * (R(1) + sr * p.x) * (R(1) + ss * p.y) * (R(1) + st * p.z);
    out.x += w * static_cast<R>(e.verts[v][0]);
    out.y += w * static_cast<R>(e.verts[v][1]);
    out.z += w * static_cast<R>(e.verts[v][2]);
  }
  return out;
}

// x(xi)  (HexElement.cu:122-139)
template <class R> V3<R> map_point(const Elem& e, const V3<R>& p) {
  if (has_ho_geom(e))
    return mk<R>(modal3<R>(e.geom[0], e.gm, p, D_NONE), modal3<R>(e.geom[1], e.gm, p, D_NONE),
                 modal3<R>(e.geom[2], e.gm, p, D_NONE));
  return map_trilinear<R>(e, p);
}

// Row-major J[row=x,y,z][col=r,s,t]  (HexElement.cu:141-206)
template <class R> void jacobian(const Elem& e, const V3<R>& p, R J[9]) {
  if (has_ho_geom(e)) {
    for (int c = 0; c < 3; ++c) {
      J[3 * c + 0] = modal3<R>(e.geom[c], e.gm, p, D_R);
      J[3 * c + 1] = modal3<R>(e.geom[c], e.gm, p, D_S);
      J[3 * c + 2] = modal3<R>(e.geom[c], e.gm, p, D_T);
    }
    return;
  }
  V3<R> dr = mk<R>(0, 0, 0), ds = mk<R>(0, 0, 0), dt = mk<R>(0, 0, 0);
  for (int v = 0; v < 8; ++v) {
    const int z = kXmlToZ[v];
    const R sr = (z & 1) ? R(1) : R(-1), ss = (z & 2) ? R(1) : R(-1), st = (z & 4) ? R(1) : R(-1);
    const R wr = R(0.125) * (R(1) + ss * p.y) * (R(1) + st * p.z) * sr;
    const R ws = R(0.125) * (R(1) + sr * p.x) * (R(1) + st * p.z) * ss;
    const R wt = R(0.125) * (R(1) + sr * p.x) * (R(1) + ss * p.y) * st;
    const R X = static_cast<R>(e.verts[v][0]), Y = static_cast<R>(e.verts[v][1]), Z = static_cast<R>(e.verts[v][2]);
    dr.x += wr * X; dr.y += wr * Y; dr.z += wr * Z;
    ds.x += ws * X; ds.y += ws * Y; ds.z += ws * Z;
    dt.x += wt * X; dt.y += wt * Y; dt.z += wt * Z;
  }
  J[0] = dr.x; J[1] = ds.x; J[2] = dt.x;
  J[3] = dr.y; J[4] = ds.y; J[5] = dt.y;
  J[6] = dr.z; J[7] = ds.z; J[8] = dt.z;
}

// Adjugate / determinant, no singular guard (HexElement.cu:208-225).
template <class R> void invert3(const R J[9], R inv[9]) {
  const R det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                J[2] * (J[3] * J[7] - J[4] * J[6]);
  const R id = R(1) / det;
  inv[0] = (J[4] * J[8] - J[5] * J[7]) * id;
  inv[1] = (J[2] * J[7] - J[1] * J[8]) * id;
  inv[2] = (J[1] * J[5] - J[2] * J[4]) * id;
  inv[3] = (J[5] * J[6] - J[3] * J[8]) * id;
  inv[4] = (J[0] * J[8] - J[2] * J[6]) * id;
  inv[5] = (J[2] * J[3] - J[0] * J[5]) * id;
  inv[6] = (J[3] * J[7] - J[4] * J[6]) * id;
  inv[7] = (J[1] * J[6] - J[0] * J[7]) * id;
  inv[8] = (J[0] * J[4] - J[1] * J[3]) * id;
}

struct Counters {
  uint64_t newton_iters = 0;   // inverse-map Newton iterations
  uint64_t face_iters = 0;     // surface Newton iterations
  uint64_t newton_solves = 0;
};

// Inverse map x(xi) = p by Newton from xi = 0: at most max_it iterations,
// converged when every |delta| < tol (HexElement.cu:227-272).
template <class R>
bool inverse_map(const Elem& e, const V3<R>& target, V3<R>& xi, Counters* cnt, int max_it = 50,
                 R tol = static_cast<R>(1e-5f)) {
  xi = mk<R>(0, 0, 0);
  if (cnt) cnt->newton_solves++;
  for (int it = 0; it < max_it; ++it) {
    if (cnt) cnt->newton_iters++;
    const V3<R> x = map_point<R>(e, xi);
    const V3<R> r = mk<R>(x.x - target.x, x.y - target.y, x.z - target.z);
    R J[9], K[9];
    jacobian<R>(e, xi, J);
    invert3<R>(J, K);
    const R d0 = K[0] * r.x + K[1] * r.y + K[2] * r.z;
    const R d1 = K[3] * r.x + K[4] * r.y + K[5] * r.z;
    const R d2 = K[6] * r.x + K[7] * r.y + K[8] * r.z;
    xi.x -= d0;
    xi.y -= d1;
    xi.z -= d2;
    if (rabs(d0) < tol && rabs(d1) < tol && rabs(d2) < tol) return true;
  }
  return false;
}

// u(xi)  (HexElement.cu:274-278)
template <class R> R field_value(const Elem& e, const V3<R>& p) { return modal3<R>(e.field, e.fm, p, D_NONE); }

// grad_xi u, one pass over the coefficients (HexElement.cu:280-306)
template <class R> V3<R> field_grad_ref(const Elem& e, const V3<R>& p) {
  V3<R> g = mk<R>(0, 0, 0);
  const float* c = e.field;
  R a[3][16], da[3][16];
  const R q[3] = {p.x, p.y, p.z};
  for (int ax = 0; ax < 3; ++ax)
    for (unsigned i = 0; i < e.fm[ax]; ++i) {
      a[ax][i] = mod_a<R>(i, q[ax]);
      da[ax][i] = mod_a_prime<R>(i, q[ax]);
    }
  int idx = 0;
  for (unsigned k = 0; k < e.fm[2]; ++k) {
    for (unsigned j = 0; j < e.fm[1]; ++j) {
      for (unsigned i = 0; i < e.fm[0]; ++i) {
        const R cv = static_cast<R>(c[idx++]);
        g.x += cv * da[0][i] * a[1][j] * a[2][k];
        g.y += cv * a[0][i] * da[1][j] * a[2][k];
        g.z += cv * a[0][i] * a[1][j] * da[2][k];
      }
    }
  }
  return g;
}

// grad_x u = J^{-T} grad_xi u  (HexElement.cu:308-330)
template <class R> V3<R> field_grad_world(const Elem& e, const V3<R>& p) {
  const V3<R> g = field_grad_ref<R>(e, p);
  R J[9], K[9];
  jacobian<R>(e, p, J);
  invert3<R>(J, K);
  return mk<R>(K[0] * g.x + K[3] * g.y + K[6] * g.z, K[1] * g.x + K[4] * g.y + K[7] * g.z,
               K[2] * g.x + K[5] * g.y + K[8] * g.z);
}

template <class R> struct Ray {
  V3<R> o, d;
};

// One sample of f(t) = u(x(t)) - iso with df/dt (RayIsosurface.cu:44-65).
template <class R> struct Sample {
  V3<R> xi;
  R f, df;
  V3<R> g;
};

template <class R>
bool sample_along(const Elem& e, const Ray<R>& ray, R t, R iso, Sample<R>& s, Counters* cnt) {
  const V3<R> p = mk<R>(ray.o.x + t * ray.d.x, ray.o.y + t * ray.d.y, ray.o.z + t * ray.d.z);
  if (!inverse_map<R>(e, p, s.xi, cnt)) return false;
  const R u = field_value<R>(e, s.xi);
  s.g = field_grad_world<R>(e, s.xi);
  s.f = u - iso;
  s.df = s.g.x * ray.d.x + s.g.y * ray.d.y + s.g.z * ray.d.z;
  return true;
}

// First sign change of f over 17 uniform samples of [t0,t1], then at most 20
// safeguarded Newton/bisection steps, done when |f| < tol
// (RayIsosurface.cu:67-188).
template <class R>
bool find_iso(const Elem& e, const Ray<R>& ray, R t0, R t1, R iso, R& t_hit, V3<R>& xi_hit, V3<R>& g_hit,
              Counters* cnt, R tol = static_cast<R>(1e-5f)) {
  const int kSeg = 16;
  bool have = false;
  R tp = t0;
  Sample<R> sp{};
  for (int i = 0; i <= kSeg; ++i) {
    const R frac = static_cast<R>(static_cast<float>(i) / static_cast<float>(kSeg));
    const R t = t0 + (t1 - t0) * frac;
    Sample<R> s{};
    if (!sample_along<R>(e, ray, t, iso, s, cnt)) continue;
    if (!have) {
      have = true;
      tp = t;
      sp = s;
      continue;
    }
    if (sp.f * s.f <= R(0)) {
      R lt = tp, rt = t;
      Sample<R> ls = sp, rs = s;
      for (int it = 0; it < 20; ++it) {
        const R mt = R(0.5) * (lt + rt);
        Sample<R> ms{};
        if (!sample_along<R>(e, ray, mt, iso, ms, cnt)) return false;
        R ct = mt;
        if (rabs(ms.df) > static_cast<R>(1e-8f)) {
          const R nt = mt - ms.f / ms.df;
          if (nt > lt && nt < rt) ct = nt;
        }
        Sample<R> cs{};
        if (!sample_along<R>(e, ray, ct, iso, cs, cnt)) {
          // keep the failed solve's xi, as the reference does
          ct = mt;
          cs.f = ms.f;
          cs.g = ms.g;
        }
        if (rabs(cs.f) < tol) {
          t_hit = ct;
          xi_hit = cs.xi;
          g_hit = cs.g;
          return true;
        }
        if (ls.f * cs.f <= R(0)) {
          rt = ct;
          rs = cs;
        } else {
          lt = ct;
          ls = cs;
        }
      }
      t_hit = R(0.5) * (lt + rt);
      xi_hit = ls.xi;
      g_hit = ls.g;
      return true;
    }
    tp = t;
    sp = s;
  }
  return false;
}

// Sampled, padded element box (FEM-AABB/high_order.h:51-113).
template <class R> void elem_box(const Elem& e, int samples, V3<R>& lo, V3<R>& hi) {
  const R big = static_cast<R>(FLT_MAX);
  lo = mk<R>(big, big, big);
  hi = mk<R>(-big, -big, -big);
  if (!has_ho_geom(e) || samples <= 1) {
    for (int v = 0; v < 8; ++v) {
      lo.x = rmin(lo.x, static_cast<R>(e.verts[v][0])); hi.x = rmax(hi.x, static_cast<R>(e.verts[v][0]));
      lo.y = rmin(lo.y, static_cast<R>(e.verts[v][1])); hi.y = rmax(hi.y, static_cast<R>(e.verts[v][1]));
      lo.z = rmin(lo.z, static_cast<R>(e.verts[v][2])); hi.z = rmax(hi.z, static_cast<R>(e.verts[v][2]));
    }
    const R pad = static_cast<R>(1e-4f);
    lo.x -= pad; lo.y -= pad; lo.z -= pad;
    hi.x += pad; hi.y += pad; hi.z += pad;
    return;
  }
  const int order = static_cast<int>(std::max(e.gm[0], std::max(e.gm[1], e.gm[2])));
  const int ns = std::max(samples, order + 2);
  for (int kz = 0; kz < ns; ++kz) {
    const R tz = R(-1) + R(2) * static_cast<R>(kz) / static_cast<R>(ns - 1);
    for (int ky = 0; ky < ns; ++ky) {
      const R sy = R(-1) + R(2) * static_cast<R>(ky) / static_cast<R>(ns - 1);
      for (int kx = 0; kx < ns; ++kx) {
        const R rx = R(-1) + R(2) * static_cast<R>(kx) / static_cast<R>(ns - 1);
        const V3<R> p = map_point<R>(e, mk<R>(rx, sy, tz));
        lo.x = rmin(lo.x, p.x); lo.y = rmin(lo.y, p.y); lo.z = rmin(lo.z, p.z);
        hi.x = rmax(hi.x, p.x); hi.y = rmax(hi.y, p.y); hi.z = rmax(hi.z, p.z);
      }
    }
  }
  const R ratio = static_cast<R>(0.15f), floor_pad = static_cast<R>(1e-3f);
  const R px = rmax((hi.x - lo.x) * ratio, floor_pad);
  const R py = rmax((hi.y - lo.y) * ratio, floor_pad);
  const R pz = rmax((hi.z - lo.z) * ratio, floor_pad);
  lo.x -= px; lo.y -= py; lo.z -= pz;
  hi.x += px; hi.y += py; hi.z += pz;
}

// Slab test clipped to [tmin,tmax] (FEM-AABB/high_order.h:115-152).
template <class R>
bool ray_box(const Ray<R>& ray, const V3<R>& lo, const V3<R>& hi, R tmin, R tmax, R& te, R& tx) {
  te = tmin;
  tx = tmax;
  for (int a = 0; a < 3; ++a) {
    const R o = comp(ray.o, a), d = comp(ray.d, a), l = comp(lo, a), h = comp(hi, a);
    if (rabs(d) < static_cast<R>(1e-8f)) {
      if (o < l || o > h) return false;
      continue;
    }
    const R inv = R(1) / d;
    R a0 = (l - o) * inv, a1 = (h - o) * inv;
    if (a0 > a1) std::swap(a0, a1);
    te = rmax(te, a0);
    tx = rmin(tx, a1);
    if (te > tx) return false;
  }
  return tx >= te;
}

// Face table: fixed axis/value and the two free axes (high_order.h:164-184).
struct FaceParam {
  int fixed;
  float val;
  int u, v;
};
inline FaceParam face_param(int f) {
  switch (f) {
    case 0: return {2, -1.f, 0, 1};
    case 1: return {1, -1.f, 0, 2};
    case 2: return {0, 1.f, 1, 2};
    case 3: return {1, 1.f, 0, 2};
    case 4: return {0, -1.f, 1, 2};
    case 5: return {2, 1.f, 0, 1};
    default: return {2, -1.f, 0, 1};
  }
}

template <class R> R ray_param_of(const Ray<R>& ray, const V3<R>& p) {
  const V3<R> d = mk<R>(p.x - ray.o.x, p.y - ray.o.y, p.z - ray.o.z);
  const R dd = dot3(ray.d, ray.d);
  return dd > R(0) ? dot3(d, ray.d) / dd : R(0);
}

// Ray against one curved face: 3x3 Newton in (u,v,tau) from the 9 seeds
// {-0.8,0,0.8}^2, at most 50 iterations, converged when max|X-Y| < tol,
// step clamp 0.25, divergence break after 5 iterations
// (FEM-AABB/high_order.h:189-304).
template <class R>
bool hit_face(const Elem& e, const Ray<R>& ray, int f, R tmin, R tmax, R& t_hit, V3<R>& xi_hit, Counters* cnt,
              R tol = static_cast<R>(1e-4f), int max_it = 50) {
  const FaceParam fp = face_param(f);
  const R seeds1[3] = {static_cast<R>(-0.8f), R(0), static_cast<R>(0.8f)};
  for (int sj = 0; sj < 3; ++sj) {
    for (int si = 0; si < 3; ++si) {
      V3<R> p = mk<R>(0, 0, 0);
      setc(p, fp.fixed, static_cast<R>(fp.val));
      setc(p, fp.u, seeds1[si]);
      setc(p, fp.v, seeds1[sj]);
      const V3<R> x0 = map_point<R>(e, p);
      R tau = rmin(rmax(ray_param_of<R>(ray, x0), tmin), tmax);
      R prev = static_cast<R>(FLT_MAX);
      for (int it = 0; it < max_it; ++it) {
        if (cnt) cnt->face_iters++;
        const V3<R> X = map_point<R>(e, p);
        const V3<R> res = mk<R>(X.x - (ray.o.x + tau * ray.d.x), X.y - (ray.o.y + tau * ray.d.y),
                                X.z - (ray.o.z + tau * ray.d.z));
        const R m = rmax(rabs(res.x), rmax(rabs(res.y), rabs(res.z)));
        if (m < tol) {
          const R pu = comp(p, fp.u), pv = comp(p, fp.v);
          const R lim = static_cast<R>(1.001f);
          if (pu >= -lim && pu <= lim && pv >= -lim && pv <= lim && tau >= tmin && tau <= tmax) {
            t_hit = tau;
            xi_hit = p;
            return true;
          }
          break;
        }
        if (it > 5 && m > prev * static_cast<R>(1.5f)) break;
        prev = m;
        R Jf[9];
        jacobian<R>(e, p, Jf);
        const V3<R> cu = mk<R>(Jf[fp.u], Jf[3 + fp.u], Jf[6 + fp.u]);
        const V3<R> cv = mk<R>(Jf[fp.v], Jf[3 + fp.v], Jf[6 + fp.v]);
        R A[9] = {cu.x, cv.x, -ray.d.x, cu.y, cv.y, -ray.d.y, cu.z, cv.z, -ray.d.z};
        R K[9];
        invert3<R>(A, K);
        const V3<R> nr = mk<R>(-res.x, -res.y, -res.z);
        const R du = K[0] * nr.x + K[1] * nr.y + K[2] * nr.z;
        const R dv = K[3] * nr.x + K[4] * nr.y + K[5] * nr.z;
        const R dtau = K[6] * nr.x + K[7] * nr.y + K[8] * nr.z;
        const R mx = rmax(rabs(du), rmax(rabs(dv), rabs(dtau)));
        const R sc = (mx > static_cast<R>(0.25f)) ? (static_cast<R>(0.25f) / mx) : R(1);
        setc(p, fp.u, comp(p, fp.u) + du * sc);
        setc(p, fp.v, comp(p, fp.v) + dv * sc);
        tau += dtau * sc;
        tau = rmin(rmax(tau, tmin), tmax);
        setc(p, fp.u, rmin(rmax(comp(p, fp.u), static_cast<R>(-1.5f)), static_cast<R>(1.5f)));
        setc(p, fp.v, rmin(rmax(comp(p, fp.v), static_cast<R>(-1.5f)), static_cast<R>(1.5f)));
        setc(p, fp.fixed, static_cast<R>(fp.val));
      }
    }
  }
  return false;
}

// Nearest face hit over the 6 faces after a box pre-test
// (FEM-AABB/high_order.h:409-465).
template <class R>
bool hit_hex(const Elem& e, const Ray<R>& ray, R tmin, R tmax, R& t_hit, V3<R>& xi_hit, int& face, Counters* cnt) {
  int samples = 0;
  if (has_ho_geom(e)) {
    const int order = static_cast<int>(std::max(e.gm[0], std::max(e.gm[1], e.gm[2])));
    samples = std::max(order + 2, 3);
  }
  V3<R> lo, hi;
  elem_box<R>(e, samples, lo, hi);
  R te, tx;
  if (!ray_box<R>(ray, lo, hi, tmin, tmax, te, tx)) return false;
  bool any = false;
  R best = tmax;
  V3<R> bxi = mk<R>(0, 0, 0);
  int bf = -1;
  for (int f = 0; f < 6; ++f) {
    R tf;
    V3<R> xf;
    if (hit_face<R>(e, ray, f, tmin, tmax, tf, xf, cnt)) {
      if (tf > tmin && tf < best) {
        best = tf;
        bxi = xf;
        bf = f;
        any = true;
      }
    }
  }
  if (any) {
    t_hit = best;
    xi_hit = bxi;
    face = bf;
  }
  return any;
}

template <class R> V3<R> normalize3(const V3<R>& v) {
  const R l = std::sqrt(dot3(v, v));
  const R s = R(1) / l;
  return mk<R>(v.x * s, v.y * s, v.z * s);
}

// Hit kinds reported per ray.
enum HitKind { HK_MISS = 0, HK_FACE = 1, HK_ISO = 2 };

template <class R> struct Hit {
  R t;
  int elem, face, kind;
  V3<R> xi, n;
  R u;
};

// Per-candidate policy of the reference's hex branch
// (FEM-AABB/raytracer.cu:184-254): iso search over the padded-box segment
// when enabled; if it finds nothing, nearest curved face. Updates `best`
// when the candidate's hit is in (0.001, best.t).
template <class R>
void visit_candidate(const Elem& e, int eidx, const Ray<R>& ray, R te, R tx, R iso, bool iso_on, Hit<R>& best,
                     Counters* cnt) {
  const R t_eps = static_cast<R>(0.001f);
  R th;
  V3<R> xi, g;
  const bool field_ok = e.field && e.fm[0] > 0 && e.fm[1] > 0 && e.fm[2] > 0;
  if (iso_on && field_ok && find_iso<R>(e, ray, te, tx, iso, th, xi, g, cnt)) {
    if (th > t_eps && th < best.t) {
      V3<R> n = normalize3(g);
      if (dot3(n, ray.d) > R(0)) n = mk<R>(-n.x, -n.y, -n.z);
      best.t = th;
      best.elem = eidx;
      best.face = -1;
      best.kind = HK_ISO;
      best.xi = xi;
      best.n = n;
      best.u = field_value<R>(e, xi);
    }
    return;
  }
  int face = -1;
  if (hit_hex<R>(e, ray, t_eps, best.t, th, xi, face, cnt)) {
    if (th > t_eps && th < best.t) {
      R J[9];
      jacobian<R>(e, xi, J);
      const V3<R> dr = mk<R>(J[0], J[3], J[6]), ds = mk<R>(J[1], J[4], J[7]), dt = mk<R>(J[2], J[5], J[8]);
      V3<R> n;
      if (rabs(xi.x) > static_cast<R>(0.9f)) n = cross3(ds, dt);
      else if (rabs(xi.y) > static_cast<R>(0.9f)) n = cross3(dr, dt);
      else n = cross3(dr, ds);
      n = normalize3(n);
      if (dot3(n, ray.d) > R(0)) n = mk<R>(-n.x, -n.y, -n.z);
      best.t = th;
      best.elem = eidx;
      best.face = face;
      best.kind = HK_FACE;
      best.xi = xi;
      best.n = n;
      best.u = field_ok ? field_value<R>(e, xi) : R(0);
    }
  }
}

}  // namespace horacle
