// Prisms, quads and curved triangles on the device: the reference's
// per-primitive maps, sampled boxes and ray intersections
// (FEM-AABB/fem/PrismElement.cu, QuadElement.cu, TriElement.cu), evaluated
// in FP32 with the reference's steps, start lists, tolerances and iteration
// caps. The translation unit that includes this header is compiled without
// multiply-add contraction, so every operation rounds as the reference's
// own FP32 host build rounds it: the start searches branch on exact values,
// and contraction would change which start converges.
#pragma once

#include <cfloat>
#include <cstdint>

#include "ho_layout.h"

namespace ho {

constexpr int kPrimPrism = 0, kPrimQuad = 1, kPrimTri = 2;
constexpr int kPrimMaxModes = 9;  // modes per direction, geometry and field

// One primitive in device memory (128 bytes). Vertices: prism 6 (quad base
// 0-3 at t = -1, top edge 4-5), quad 4 (vertex v at r = +-1 by bit 0 and
// s = +-1 by bit 1), triangle 3. Modes packed x | y << 8 | z << 16 (0 =
// linear geometry / no field); goff / foff are float offsets into the
// primitive geometry and field pools (geometry: x, y, z blocks back to back).
struct alignas(16) PrimRec {
  float v[18];
  float lo[3], hi[3];  // sampled box
  int32_t kind, local;  // kind and index among the primitives of that kind
  uint32_t gm, fm;
  int64_t goff, foff;
};
static_assert(sizeof(PrimRec) == 128, "PrimRec is two 64-byte lines");

__host__ __device__ inline unsigned pmode(uint32_t packed, int a) { return (packed >> (8 * a)) & 0xffu; }

// Coefficients in one component block.
__host__ __device__ inline int prim_block(int kind, uint32_t m) {
  const int mx = static_cast<int>(pmode(m, 0)), my = static_cast<int>(pmode(m, 1)), mz = static_cast<int>(pmode(m, 2));
  if (kind == kPrimQuad) return mx * my;
  const int top = kind == kPrimPrism ? mz : my;
  int n = 0;
  for (int i = 0; i < mx; ++i) n += top > i ? top - i : 0;
  return kind == kPrimPrism ? n * my : n;
}

// ---------------------------------------------------------------------------
// 1-D bases: Jacobi recurrence, Modified-A and Modified-B and derivatives
// (FEM-AABB/fem/ModalBasis.cuh), same grouping of operations.
// ---------------------------------------------------------------------------
__device__ inline float pr_jacobi(int n, float a, float b, float x) {
  if (n == 0) return 1.0f;
  const float p1 = 0.5f * ((2.0f + a + b) * x + (a - b));
  if (n == 1) return p1;
  float pm2 = 1.0f, pm1 = p1, p = 0.0f;
  for (int k = 2; k <= n; ++k) {
    const float kf = static_cast<float>(k);
    const float s = 2.0f * kf + a + b;
    const float den = 2.0f * kf * (kf + a + b) * (s - 2.0f);
    const float up = (s - 1.0f) * (s * (s - 2.0f) * x + (a * a - b * b)) * pm1;
    const float dn = 2.0f * (kf + a - 1.0f) * (kf + b - 1.0f) * s * pm2;
    p = (up - dn) / den;
    pm2 = pm1;
    pm1 = p;
  }
  return p;
}

__device__ inline float pr_jacobi_d(int n, float a, float b, float x) {
  if (n == 0) return 0.0f;
  return 0.5f * (static_cast<float>(n) + a + b + 1.0f) * pr_jacobi(n - 1, a + 1.0f, b + 1.0f, x);
}

__device__ inline float pr_a(unsigned i, float x) {
  if (i == 0) return 0.5f * (1.0f - x);
  if (i == 1) return 0.5f * (1.0f + x);
  return 0.25f * (1.0f - x * x) * pr_jacobi(static_cast<int>(i) - 2, 1.0f, 1.0f, x);
}

__device__ inline float pr_a_d(unsigned i, float x) {
  if (i == 0) return -0.5f;
  if (i == 1) return 0.5f;
  const int n = static_cast<int>(i) - 2;
  return -0.5f * x * pr_jacobi(n, 1.0f, 1.0f, x) + 0.25f * (1.0f - x * x) * pr_jacobi_d(n, 1.0f, 1.0f, x);
}

__device__ inline float pr_pow(float b, unsigned p) {
  float r = 1.0f;
  for (unsigned i = 0; i < p; ++i) r *= b;
  return r;
}

__device__ inline float pr_b(unsigned i, unsigned j, float x) {
  if (i == 0) return pr_a(j, x);
  float v = pr_pow((1.0f - x) * 0.5f, i);
  if (j == 0) return v;
  v *= 0.5f * (1.0f + x);
  v *= pr_jacobi(static_cast<int>(j) - 1, 2.0f * static_cast<float>(i) - 1.0f, 1.0f, x);
  return v;
}

__device__ inline float pr_b_d(unsigned i, unsigned j, float x) {
  if (i == 0) return pr_a_d(j, x);
  if (j == 0) {
    float v = -static_cast<float>(i);
    v *= pr_pow(1.0f - x, i - 1);
    v *= pr_pow(0.5f, i);
    return v;
  }
  const float a = 2.0f * static_cast<float>(i) - 1.0f;
  const float scale = pr_pow(0.5f, i + 1);
  const float p = pr_jacobi(static_cast<int>(j) - 1, a, 1.0f, x);
  const float dp = pr_jacobi_d(static_cast<int>(j) - 1, a, 1.0f, x);
  const float t1 = pr_pow(1.0f - x, i) * p;
  const float t2 = static_cast<float>(i) * pr_pow(1.0f - x, i - 1) * (1.0f + x) * p;
  const float t3 = pr_pow(1.0f - x, i) * (1.0f + x) * dp;
  return scale * (t1 - t2 + t3);
}

// ---------------------------------------------------------------------------
// Geometry: point and tangents of a primitive at reference coordinates.
// ---------------------------------------------------------------------------
struct PrimView {
  const PrimRec* __restrict__ rec;
  const float* __restrict__ geom;
  const float* __restrict__ field;
};

__device__ inline float3 pr_vert(const PrimRec& p, int v) { return make_float3(p.v[3 * v], p.v[3 * v + 1], p.v[3 * v + 2]); }

__device__ inline bool pr_curved(const PrimRec& p) { return p.goff >= 0 && p.gm != 0; }

// Modal point (and, when tan != nullptr, the r, s, t tangents) of a curved
// primitive. Sum orders: prism i, j, k; quad j, i; triangle i, j. Each 1-D
// basis value is computed once per evaluation and reused across the other
// indices; the values and the order of the sums are those of evaluating
// every term afresh. Out of line, like the other solver routines below: one
// copy of each in the kernel keeps its code within the instruction cache.
__device__ __noinline__ void pr_modal_geom(const PrimRec& p, const float* __restrict__ pool, float3 x, float3& X,
                                           float3* tan) {
  const float* c = pool + p.goff;
  const int blk = prim_block(p.kind, p.gm);
  const unsigned mx = pmode(p.gm, 0), my = pmode(p.gm, 1), mz = pmode(p.gm, 2);
  float v[3] = {0.f, 0.f, 0.f}, dr[3] = {0.f, 0.f, 0.f}, ds[3] = {0.f, 0.f, 0.f}, dt[3] = {0.f, 0.f, 0.f};
  float ar[kPrimMaxModes], dar[kPrimMaxModes], bs[kPrimMaxModes], dbs[kPrimMaxModes];
  for (unsigned i = 0; i < mx; ++i) {
    ar[i] = pr_a(i, x.x);
    dar[i] = tan ? pr_a_d(i, x.x) : 0.f;
  }
  int idx = 0;
  if (p.kind == kPrimPrism) {
    for (unsigned j = 0; j < my; ++j) {
      bs[j] = pr_a(j, x.y);
      dbs[j] = tan ? pr_a_d(j, x.y) : 0.f;
    }
    float bt[kPrimMaxModes], dbt[kPrimMaxModes];
    for (unsigned i = 0; i < mx; ++i) {
      const float ri = ar[i], dri = dar[i];
      const unsigned top = mz > i ? mz - i : 0;
      for (unsigned k = 0; k < top; ++k) {
        bt[k] = pr_b(i, k, x.z);
        dbt[k] = tan ? pr_b_d(i, k, x.z) : 0.f;
      }
      for (unsigned j = 0; j < my; ++j) {
        const float sj = bs[j], dsj = dbs[j];
        for (unsigned k = 0; k < top; ++k, ++idx) {
          const float tk = bt[k];
          const float dtk = dbt[k];
          for (int a = 0; a < 3; ++a) {
            const float cf = __ldg(c + a * blk + idx);
            v[a] += cf * ri * sj * tk;
            if (tan) {
              dr[a] += cf * dri * sj * tk;
              ds[a] += cf * ri * dsj * tk;
              dt[a] += cf * ri * sj * dtk;
            }
          }
        }
      }
    }
  } else if (p.kind == kPrimQuad) {
    for (unsigned j = 0; j < my; ++j) {
      const float sj = pr_a(j, x.y), dsj = tan ? pr_a_d(j, x.y) : 0.f;
      for (unsigned i = 0; i < mx; ++i, ++idx) {
        const float ri = ar[i], dri = dar[i];
        for (int a = 0; a < 3; ++a) {
          const float cf = __ldg(c + a * blk + idx);
          v[a] += cf * ri * sj;
          if (tan) {
            dr[a] += cf * dri * sj;
            ds[a] += cf * ri * dsj;
          }
        }
      }
    }
  } else {
    for (unsigned i = 0; i < mx; ++i) {
      const float ai = ar[i], dai = dar[i];
      const unsigned top = my > i ? my - i : 0;
      for (unsigned j = 0; j < top; ++j, ++idx) {
        const float bj = pr_b(i, j, x.y);
        const float dbj = tan ? pr_b_d(i, j, x.y) : 0.f;
        for (int a = 0; a < 3; ++a) {
          const float cf = __ldg(c + a * blk + idx);
          v[a] += cf * ai * bj;
          if (tan) {
            dr[a] += cf * dai * bj;
            ds[a] += cf * ai * dbj;
          }
        }
      }
    }
  }
  X = make_float3(v[0], v[1], v[2]);
  if (tan) {
    tan[0] = make_float3(dr[0], dr[1], dr[2]);
    tan[1] = make_float3(ds[0], ds[1], ds[2]);
    tan[2] = make_float3(dt[0], dt[1], dt[2]);
  }
}

// Clamped barycentric (u, v) of a triangle's (r, s) (TriElement.cu:17-31).
__device__ inline void pr_bary(float r, float s, float& u, float& v) {
  u = fminf(fmaxf(0.5f * (r + 1.0f), 0.0f), 1.0f);
  v = fminf(fmaxf(0.5f * (s + 1.0f), 0.0f), 1.0f);
  if (u + v > 1.0f) {
    const float ex = u + v - 1.0f;
    u = fmaxf(u - 0.5f * ex, 0.0f);
    v = fmaxf(v - 0.5f * ex, 0.0f);
  }
}

// Linear point and tangents. The prism's t tangent carries the reference's
// extra 0.5 (1 + r) dr term (PrismElement.cu:264-270).
__device__ __noinline__ void pr_linear_geom(const PrimRec& p, float3 x, float3& X, float3* tan) {
  float acc[3] = {0.f, 0.f, 0.f}, dr[3] = {0.f, 0.f, 0.f}, ds[3] = {0.f, 0.f, 0.f}, dt[3] = {0.f, 0.f, 0.f};
  if (p.kind == kPrimPrism) {
    const float rm = 1.0f - x.x, rp = 1.0f + x.x, sm = 1.0f - x.y, sp = 1.0f + x.y, tm = 1.0f - x.z, tp = 1.0f + x.z;
    const float w[6] = {0.125f * (rm * sm * tm), 0.125f * (rp * sm * tm), 0.125f * (rp * sp * tm),
                        0.125f * (rm * sp * tm), 0.25f * (sm * tp), 0.25f * (sp * tp)};
    for (int vtx = 0; vtx < 6; ++vtx)
      for (int a = 0; a < 3; ++a) acc[a] += w[vtx] * p.v[3 * vtx + a];
    if (tan) {
      for (int a = 0; a < 3; ++a) {
        const float* q = p.v + a;
        const float v0 = q[0], v1 = q[3], v2 = q[6], v3 = q[9], v4 = q[12], v5 = q[15];
        dr[a] = 0.25f * (-sm * v0 + sm * v1 + sp * v2 - sp * v3);
        ds[a] = 0.125f * (-rm * v0 - rp * v1 + rp * v2 + rm * v3) * tm + 0.25f * (-tp * v4 + tp * v5);
        dt[a] = 0.125f * (-rm * sm * v0 - rp * sm * v1 - rp * sp * v2 - rm * sp * v3) + 0.25f * (sm * v4 + sp * v5) +
                0.5f * rp * dr[a];
      }
    }
  } else if (p.kind == kPrimQuad) {
    for (int vtx = 0; vtx < 4; ++vtx) {
      const float sr = (vtx & 1) ? 1.0f : -1.0f, ss = (vtx & 2) ? 1.0f : -1.0f;
      const float w = 0.25f * (1.0f + sr * x.x) * (1.0f + ss * x.y);
      const float wr = 0.25f * sr * (1.0f + ss * x.y), ws = 0.25f * ss * (1.0f + sr * x.x);
      for (int a = 0; a < 3; ++a) {
        acc[a] += w * p.v[3 * vtx + a];
        dr[a] += wr * p.v[3 * vtx + a];
        ds[a] += ws * p.v[3 * vtx + a];
      }
    }
  } else {
    float u, v;
    pr_bary(x.x, x.y, u, v);
    const float w0 = fmaxf(0.0f, 1.0f - u - v);
    for (int a = 0; a < 3; ++a) {
      acc[a] += w0 * p.v[a];
      acc[a] += u * p.v[3 + a];
      acc[a] += v * p.v[6 + a];
      dr[a] = 0.5f * (p.v[3 + a] - p.v[a]);
      ds[a] = 0.5f * (p.v[6 + a] - p.v[a]);
    }
  }
  X = make_float3(acc[0], acc[1], acc[2]);
  if (tan) {
    tan[0] = make_float3(dr[0], dr[1], dr[2]);
    tan[1] = make_float3(ds[0], ds[1], ds[2]);
    tan[2] = make_float3(dt[0], dt[1], dt[2]);
  }
}

__device__ inline void pr_geom(const PrimRec& p, const float* __restrict__ pool, float3 x, float3& X, float3* tan) {
  if (pr_curved(p)) pr_modal_geom(p, pool, x, X, tan);
  else pr_linear_geom(p, x, X, tan);
}

__device__ inline float3 pr_point(const PrimRec& p, const float* __restrict__ pool, float3 x) {
  float3 X;
  pr_geom(p, pool, x, X, nullptr);
  return X;
}

// Work of one query's primitive visits: solver iterations and algorithmic
// FP32 flops. A curved evaluation costs (6 + b) flops per coefficient and
// output (b = 2 basis products in 3-D, 1 in 2-D; outputs: the point plus 3 or
// 2 tangents when asked for); a linear one a fixed count per kind.
struct PrimWork {
  uint32_t iters = 0;
  unsigned long long flops = 0;
};

__device__ inline unsigned pr_geom_flops(const PrimRec& p, bool tan) {
  if (pr_curved(p)) {
    const unsigned outs = 1u + (tan ? (p.kind == kPrimPrism ? 3u : 2u) : 0u);
    return static_cast<unsigned>(prim_block(p.kind, p.gm)) * (p.kind == kPrimPrism ? 8u : 7u) * outs;
  }
  if (p.kind == kPrimPrism) return tan ? 170u : 60u;
  if (p.kind == kPrimQuad) return tan ? 100u : 40u;
  return tan ? 47u : 35u;
}

// Field value (0 without a field).
__device__ __noinline__ float pr_field(const PrimRec& p, const float* __restrict__ pool, float3 x) {
  if (p.foff < 0) return 0.f;
  const float* c = pool + p.foff;
  const unsigned mx = pmode(p.fm, 0), my = pmode(p.fm, 1), mz = pmode(p.fm, 2);
  float sum = 0.f;
  int idx = 0;
  if (p.kind == kPrimPrism) {
    if (mx == 0 || my == 0 || mz == 0) return 0.f;
    for (unsigned i = 0; i < mx; ++i)
      for (unsigned j = 0; j < my; ++j) {
        const unsigned top = mz > i ? mz - i : 0;
        for (unsigned k = 0; k < top; ++k) sum += __ldg(c + idx++) * pr_a(i, x.x) * pr_a(j, x.y) * pr_b(i, k, x.z);
      }
  } else if (p.kind == kPrimQuad) {
    for (unsigned j = 0; j < my; ++j)
      for (unsigned i = 0; i < mx; ++i) sum += __ldg(c + idx++) * pr_a(i, x.x) * pr_a(j, x.y);
  } else {
    if (mx == 0 || my == 0) return 0.f;
    for (unsigned i = 0; i < mx; ++i) {
      const unsigned top = my > i ? my - i : 0;
      for (unsigned j = 0; j < top; ++j) sum += __ldg(c + idx++) * pr_a(i, x.x) * pr_b(i, j, x.y);
    }
  }
  return sum;
}

// Sampled box: the vertices plus a 4^3 (prism) / 4^2 (quad) grid, or, for a
// curved triangle, the 28 points of a 6-per-edge triangular grid.
__device__ void pr_box(const PrimRec& p, const float* __restrict__ pool, float lo[3], float hi[3]) {
  for (int a = 0; a < 3; ++a) {
    lo[a] = FLT_MAX;
    hi[a] = -FLT_MAX;
  }
  auto grow = [&](float3 q) {
    lo[0] = fminf(lo[0], q.x); lo[1] = fminf(lo[1], q.y); lo[2] = fminf(lo[2], q.z);
    hi[0] = fmaxf(hi[0], q.x); hi[1] = fmaxf(hi[1], q.y); hi[2] = fmaxf(hi[2], q.z);
  };
  const int nv = p.kind == kPrimPrism ? 6 : (p.kind == kPrimQuad ? 4 : 3);
  for (int v = 0; v < nv; ++v) grow(pr_vert(p, v));
  if (p.kind == kPrimTri) {
    if (!pr_curved(p)) return;
    for (int i = 0; i <= 6; ++i)
      for (int j = 0; j <= 6 - i; ++j) {
        const float u = static_cast<float>(i) / 6.0f, v = static_cast<float>(j) / 6.0f;
        grow(pr_point(p, pool, make_float3(2.0f * u - 1.0f, 2.0f * v - 1.0f, 0.f)));
      }
    return;
  }
  const int nk = p.kind == kPrimPrism ? 4 : 1;
  for (int k = 0; k < nk; ++k)
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 4; ++i) {
        const float w = p.kind == kPrimPrism ? -1.0f + 2.0f * static_cast<float>(k) / 3.0f : 0.f;
        grow(pr_point(p, pool,
                      make_float3(-1.0f + 2.0f * static_cast<float>(i) / 3.0f, -1.0f + 2.0f * static_cast<float>(j) / 3.0f,
                                  w)));
      }
}

// ---------------------------------------------------------------------------
// Ray intersections
// ---------------------------------------------------------------------------
__device__ inline float pr_dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ inline float3 pr_sub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ inline float3 pr_at(float3 o, float3 d, float t) {
  return make_float3(o.x + t * d.x, o.y + t * d.y, o.z + t * d.z);
}
__device__ inline float pr_param(float3 o, float3 d, float3 q) {
  const float dd = pr_dot(d, d);
  return dd > 0.0f ? pr_dot(pr_sub(q, o), d) / dd : 0.0f;
}
__device__ inline float pr_maxabs(float3 v) { return fmaxf(fabsf(v.x), fmaxf(fabsf(v.y), fabsf(v.z))); }
__device__ inline float3 pr_cross(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ inline float3 pr_unit(float3 v) {
  const float k = 1.0f / sqrtf(pr_dot(v, v));
  return make_float3(v.x * k, v.y * k, v.z * k);
}

// Slab test of a ray against [lo, hi] on [tmin, tmax] (entry, exit).
__device__ inline bool pr_slab(float3 o, float3 d, const float lo[3], const float hi[3], float tmin, float tmax,
                               float& te, float& tx) {
  te = tmin;
  tx = tmax;
  const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
  for (int a = 0; a < 3; ++a) {
    if (fabsf(dd[a]) < 1e-8f) {
      if (oo[a] < lo[a] || oo[a] > hi[a]) return false;
      continue;
    }
    const float inv = 1.0f / dd[a];
    float a0 = (lo[a] - oo[a]) * inv, a1 = (hi[a] - oo[a]) * inv;
    if (a0 > a1) {
      const float s = a0;
      a0 = a1;
      a1 = s;
    }
    te = fmaxf(te, a0);
    tx = fminf(tx, a1);
    if (te > tx) return false;
  }
  return tx >= te;
}

// Adjugate solve of the 3x3 system A x = b (rows of A); false if |det| < 1e-12.
__device__ inline bool pr_solve3(const float A[9], float3 b, float3& x) {
  const float det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                    A[2] * (A[3] * A[7] - A[4] * A[6]);
  if (fabsf(det) < 1e-12f) return false;
  const float id = 1.0f / det;
  const float i0 = (A[4] * A[8] - A[5] * A[7]) * id, i1 = (A[2] * A[7] - A[1] * A[8]) * id,
              i2 = (A[1] * A[5] - A[2] * A[4]) * id, i3 = (A[5] * A[6] - A[3] * A[8]) * id,
              i4 = (A[0] * A[8] - A[2] * A[6]) * id, i5 = (A[2] * A[3] - A[0] * A[5]) * id,
              i6 = (A[3] * A[7] - A[4] * A[6]) * id, i7 = (A[1] * A[6] - A[0] * A[7]) * id,
              i8 = (A[0] * A[4] - A[1] * A[3]) * id;
  x = make_float3(i0 * b.x + i1 * b.y + i2 * b.z, i3 * b.x + i4 * b.y + i5 * b.z, i6 * b.x + i7 * b.y + i8 * b.z);
  return true;
}

// Prism (PrismElement.cu:456-532): from each of 7 starts, Newton steps
// J dx = x(rst) - (closest ray point), at most 60; accepted within 1e-5 and
// inside [-1.05, 1.05]^3; a start ends when the closest ray point leaves
// the box segment or J is singular.
__device__ __noinline__ bool pr_hit_prism(const PrimRec& p, const float* __restrict__ pool, float3 o, float3 d, float tmin,
                             float tmax, float& th, float3& xh, PrimWork& w) {
  float enter, exit;
  if (!pr_slab(o, d, p.lo, p.hi, tmin, tmax, enter, exit)) return false;
  const float seeds[7][3] = {{0.f, 0.f, 0.f},     {-0.5f, -0.5f, -0.5f}, {0.5f, -0.5f, -0.5f}, {0.f, 0.5f, -0.5f},
                             {-0.5f, 0.f, 0.5f}, {0.5f, 0.f, 0.5f},     {0.f, 0.5f, 0.5f}};
  for (int sd = 0; sd < 7; ++sd) {
    float3 x = make_float3(seeds[sd][0], seeds[sd][1], seeds[sd][2]);
    for (int it = 0; it < 60; ++it) {
      ++w.iters;
      w.flops += pr_geom_flops(p, true) + 81u;  // + closest point, residual, 3x3 solve
      float3 X, tan[3];
      pr_geom(p, pool, x, X, tan);
      const float tau = pr_param(o, d, X);
      if (tau < enter || tau > exit) break;
      const float3 res = pr_sub(X, pr_at(o, d, tau));
      if (pr_maxabs(res) < 1e-5f && x.x >= -1.05f && x.x <= 1.05f && x.y >= -1.05f && x.y <= 1.05f &&
          x.z >= -1.05f && x.z <= 1.05f) {
        th = tau;
        xh = x;
        return true;
      }
      const float A[9] = {tan[0].x, tan[1].x, tan[2].x, tan[0].y, tan[1].y, tan[2].y, tan[0].z, tan[1].z, tan[2].z};
      float3 dx;
      if (!pr_solve3(A, res, dx)) break;
      x = make_float3(x.x - dx.x, x.y - dx.y, x.z - dx.z);
    }
  }
  return false;
}

// Gauss-Newton projection of q onto a surface primitive from (r0, s0).
__device__ __noinline__ bool pr_project(const PrimRec& p, const float* __restrict__ pool, float3 q, float r0, float s0, float& r,
                           float& s, int max_it, float tol, PrimWork& w) {
  r = r0;
  s = s0;
  for (int it = 0; it < max_it; ++it) {
    ++w.iters;
    w.flops += pr_geom_flops(p, true) + 39u;  // + metric tensor, 2x2 solve
    float3 X, tan[3];
    pr_geom(p, pool, make_float3(r, s, 0.f), X, tan);
    const float3 diff = pr_sub(X, q);
    const float g00 = pr_dot(tan[0], tan[0]), g01 = pr_dot(tan[0], tan[1]), g11 = pr_dot(tan[1], tan[1]);
    const float det = g00 * g11 - g01 * g01;
    if (fabsf(det) < 1e-10f) return false;
    const float id = 1.0f / det;
    const float b0 = pr_dot(tan[0], diff), b1 = pr_dot(tan[1], diff);
    const float dr = id * (g11 * b0 - g01 * b1);
    const float ds = id * (-g01 * b0 + g00 * b1);
    r -= dr;
    s -= ds;
    if (fabsf(dr) < tol && fabsf(ds) < tol) return true;
  }
  return false;
}

// Does q lie on the surface? Quad (QuadElementContainsPoint, 9 starts, 40
// steps at 1e-4, inside [-1.05, 1.05]^2, maps back within 5e-4); triangle
// (4 starts of 30 steps at 1e-4, then the clamped-barycentric inside test).
__device__ __noinline__ bool pr_contains(const PrimRec& p, const float* __restrict__ pool, float3 q, float& r_out, float& s_out,
                            PrimWork& w) {
  if (p.kind == kPrimQuad) {
    const float seeds[9][2] = {{0.f, 0.f},     {-0.5f, -0.5f}, {0.5f, -0.5f}, {-0.5f, 0.5f}, {0.5f, 0.5f},
                               {-0.9f, -0.9f}, {0.9f, -0.9f},  {-0.9f, 0.9f}, {0.9f, 0.9f}};
    for (int sd = 0; sd < 9; ++sd) {
      float r, s;
      if (!pr_project(p, pool, q, seeds[sd][0], seeds[sd][1], r, s, 40, 1e-4f, w)) continue;
      if (r < -1.05f || r > 1.05f || s < -1.05f || s > 1.05f) continue;
      w.flops += pr_geom_flops(p, false);
      const float3 X = pr_point(p, pool, make_float3(r, s, 0.f));
      if (fabsf(X.x - q.x) > 5e-4f || fabsf(X.y - q.y) > 5e-4f || fabsf(X.z - q.z) > 5e-4f) continue;
      r_out = r;
      s_out = s;
      return true;
    }
    return false;
  }
  const float seeds[4][2] = {{0.f, 0.f}, {-0.5f, -0.5f}, {0.5f, -0.5f}, {0.f, 0.5f}};
  float r = 0.f, s = 0.f;
  bool ok = false;
  for (int sd = 0; sd < 4 && !ok; ++sd) ok = pr_project(p, pool, q, seeds[sd][0], seeds[sd][1], r, s, 30, 1e-4f, w);
  if (!ok) return false;
  float u, v;
  pr_bary(r, s, u, v);
  const float w0 = 1.0f - u - v;
  if (!(u >= -1e-3f && v >= -1e-3f && w0 >= -1e-3f)) return false;
  r_out = r;
  s_out = s;
  return true;
}

// Quad / triangle (QuadElement.cu:402-527, TriElement.cu:224-497): a start
// from the first of 11 (quad) / 9 (triangle) box-segment points on the
// surface, else the vertex plane, else the segment middle; then Newton on
// (r, s, t) for x(r, s) = o + t d, at most 40 steps at 1e-5.
__device__ __noinline__ bool pr_hit_surface(const PrimRec& p, const float* __restrict__ pool, float3 o, float3 d, float tmin,
                               float tmax, float& th, float3& xh, PrimWork& w) {
  float enter, exit;
  if (!pr_slab(o, d, p.lo, p.hi, tmin, tmax, enter, exit)) return false;
  const bool quad = p.kind == kPrimQuad;
  const int n = quad ? 10 : 8;
  float t = 0.f, r = 0.f, s = 0.f;
  bool started = false;
  for (int i = 0; i <= n && !started; ++i) {
    const float u = static_cast<float>(i) / static_cast<float>(n);
    float rr, ss;
    if (pr_contains(p, pool, pr_at(o, d, enter + (exit - enter) * u), rr, ss, w)) {
      r = rr;
      s = ss;
      t = pr_param(o, d, pr_point(p, pool, make_float3(r, s, 0.f)));
      started = true;
    }
  }
  if (!started) {
    const float3 a = pr_vert(p, 0), b = pr_vert(p, 1), c = pr_vert(p, quad ? 3 : 2);
    const float3 nrm = pr_unit(pr_cross(pr_sub(b, a), pr_sub(c, a)));
    const float den = pr_dot(nrm, d);
    const float mid = 0.5f * (enter + exit);
    if (quad) {
      t = mid;
      if (fabsf(den) > 1e-6f) {
        float tp = pr_dot(nrm, pr_sub(a, o)) / den;
        if (tp < enter || tp > exit) tp = mid;
        float rr, ss;
        if (pr_contains(p, pool, pr_at(o, d, tp), rr, ss, w)) {
          r = rr;
          s = ss;
          t = pr_param(o, d, pr_point(p, pool, make_float3(r, s, 0.f)));
        }
      }
    } else {
      float tp = mid;
      if (fabsf(den) > 1e-6f) {
        const float q = pr_dot(nrm, pr_sub(a, o)) / den;
        if (q >= enter && q <= exit) tp = q;
      }
      float rr, ss;
      if (pr_contains(p, pool, pr_at(o, d, tp), rr, ss, w)) {
        r = rr;
        s = ss;
      }
      t = pr_param(o, d, pr_point(p, pool, make_float3(r, s, 0.f)));
    }
  }
  for (int it = 0; it < 40; ++it) {
    ++w.iters;
    w.flops += pr_geom_flops(p, true) + 69u;  // + ray point, residual, 3x3 solve
    float3 X, tan[3];
    pr_geom(p, pool, make_float3(r, s, 0.f), X, tan);
    const float3 res = pr_sub(pr_at(o, d, t), X);
    const bool inside = !quad || (r >= -1.02f && r <= 1.02f && s >= -1.02f && s <= 1.02f);
    if (pr_maxabs(res) < 1e-5f && inside && t >= tmin && t <= tmax) {
      th = t;
      xh = make_float3(r, s, 0.f);
      return true;
    }
    const float A[9] = {-tan[0].x, -tan[1].x, d.x, -tan[0].y, -tan[1].y, d.y, -tan[0].z, -tan[1].z, d.z};
    float3 dx;
    if (!pr_solve3(A, make_float3(-res.x, -res.y, -res.z), dx)) return false;
    r += dx.x;
    s += dx.y;
    t += dx.z;
    if (quad && (t < tmin || t > tmax)) return false;
  }
  return false;
}

__device__ inline bool pr_hit(const PrimRec& p, const float* __restrict__ pool, float3 o, float3 d, float tmin,
                              float tmax, float& th, float3& xh, PrimWork& w) {
  return p.kind == kPrimPrism ? pr_hit_prism(p, pool, o, d, tmin, tmax, th, xh, w)
                              : pr_hit_surface(p, pool, o, d, tmin, tmax, th, xh, w);
}

// Normal at a hit: unit cross product of the r and s tangents turned against
// the ray, then negated once more unless strictly against it (the
// reference's HitRecord::set_face_normal).
__device__ __noinline__ float3 pr_normal(const PrimRec& p, const float* __restrict__ pool, float3 x, float3 d) {
  float3 X, tan[3];
  pr_geom(p, pool, x, X, tan);
  float3 n = pr_unit(pr_cross(tan[0], tan[1]));
  if (pr_dot(n, d) > 0.0f) n = make_float3(-n.x, -n.y, -n.z);
  if (!(pr_dot(d, n) < 0.0f)) n = make_float3(-n.x, -n.y, -n.z);
  return n;
}

}  // namespace ho
