// Device-side element math for curved hexahedra with Modified-A modal
// geometry and field. All arithmetic FP32; templated on N = modes per
// direction so every tensor loop unrolls.
//
// Algorithm steps follow the reference's per-element functions
// (paths relative to the reference project root):
//   basis            FEM-AABB/fem/ModalBasis.cuh:16-70
//   map / Jacobian   FEM-AABB/fem/HexElement.cu:8-206  (here sum-factorised)
//   inverse map      FEM-AABB/fem/HexElement.cu:227-272
//   field, gradient  FEM-AABB/fem/HexElement.cu:274-330
//   isosurface scan  FEM-AABB/fem/RayIsosurface.cu:44-188
//   padded box       FEM-AABB/high_order.h:51-113
//   slab test        FEM-AABB/high_order.h:115-152
//   face Newton      FEM-AABB/high_order.h:164-304
//   nearest face     FEM-AABB/high_order.h:409-465
//   hex hit policy   FEM-AABB/raytracer.cu:184-254
#pragma once

#include <cfloat>
#include <cstdint>

#include "ho_layout.h"

namespace ho {

// ---------------------------------------------------------------------------
// Work counters kept in registers per thread and flushed once per thread.
// ---------------------------------------------------------------------------
struct Work {
  uint32_t cand = 0, geom = 0, map = 0, field = 0, newton = 0, face = 0, culled = 0, nodes = 0, restarts = 0;
  uint32_t accepted = 0, rejected = 0;
  // SM cycles by phase (warp kernels, counted on lane 0): traversal, isosurface
  // scan, bracket refinement, face search
  unsigned long long cyc[4] = {0, 0, 0, 0};
  // round kernel: loop steps and busy lanes over them (counted on lane 0)
  unsigned long long steps = 0, lanes = 0;
  // round kernel: algorithmic FP32 flops of the evaluations and solves done
  unsigned long long flops = 0;
};

// Algorithmic flops of one sum-factorised point evaluation of `comps`
// components (value and three partials each) at n modes per direction: the
// 1-D basis values and derivatives (3 x 8n) plus 2(2n^3 + 3n^2 + 4n) per
// component; and of one 3x3 Newton solve and update.
__host__ __device__ constexpr unsigned long long eval_flops(int n, int comps) {
  return 3ull * 8 * n + 2ull * comps * (2ull * n * n * n + 3ull * n * n + 4ull * n);
}
constexpr unsigned long long kSolveFlops = 60;

// ---------------------------------------------------------------------------
// 1-D Modified-A basis: phi_0 = (1-x)/2, phi_1 = (1+x)/2,
// phi_i = (1-x^2)/4 * P^{(1,1)}_{i-2}(x). P^{(1,1)} by the three-term
// recurrence P_m = A_m x P_{m-1} - B_m P_{m-2}, A_m = (2m+1)(m+1)/(m(m+2)),
// B_m = (m+1)/(m+2), P_0 = 1, P_1 = 2x (the alpha = beta = 1 case of the
// general recurrence in ModalBasis.cuh:16-41); derivatives by differentiating
// the same recurrence.
// ---------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void basis_val(float x, float (&a)[N]) {
  a[0] = 0.5f * (1.0f - x);
  if (N > 1) a[1] = 0.5f * (1.0f + x);
  const float w = 0.25f * (1.0f - x * x);
  float pm2 = 1.0f, pm1 = 2.0f * x;
#pragma unroll
  for (int i = 2; i < N; ++i) {
    const int m = i - 2;
    float p;
    if (m == 0) p = 1.0f;
    else if (m == 1) p = pm1;
    else {
      const float A = float((2 * m + 1) * (m + 1)) / float(m * (m + 2));
      const float B = float(m + 1) / float(m + 2);
      p = A * x * pm1 - B * pm2;
      pm2 = pm1;
      pm1 = p;
    }
    a[i] = w * p;
  }
}

template <int N>
__device__ __forceinline__ void basis_val_der(float x, float (&a)[N], float (&d)[N]) {
  a[0] = 0.5f * (1.0f - x);
  d[0] = -0.5f;
  if (N > 1) {
    a[1] = 0.5f * (1.0f + x);
    d[1] = 0.5f;
  }
  const float w = 0.25f * (1.0f - x * x);
  const float hx = -0.5f * x;
  float pm2 = 1.0f, pm1 = 2.0f * x, qm2 = 0.0f, qm1 = 2.0f;
#pragma unroll
  for (int i = 2; i < N; ++i) {
    const int m = i - 2;
    float p, q;
    if (m == 0) {
      p = 1.0f;
      q = 0.0f;
    } else if (m == 1) {
      p = pm1;
      q = qm1;
    } else {
      const float A = float((2 * m + 1) * (m + 1)) / float(m * (m + 2));
      const float B = float(m + 1) / float(m + 2);
      p = A * x * pm1 - B * pm2;
      q = A * (pm1 + x * qm1) - B * qm2;
      pm2 = pm1;
      pm1 = p;
      qm2 = qm1;
      qm1 = q;
    }
    a[i] = w * p;
    d[i] = hx * p + w * q;
  }
}

// ---------------------------------------------------------------------------
// Sum-factorised tensor contractions. Coefficient index ((k*N)+j)*N+i,
// i fastest (HexElement.cu:14-26). One component per call.
//
// Code size matters more than call overhead here: a fully unrolled N^3
// contraction is thousands of instructions, and inlining it at every call
// site overflows the instruction cache. So the i and j loops are unrolled
// (basis values in registers), the k loop is rolled (its basis values come
// from the caller's per-lane local array), and the routines are out of line.
// ---------------------------------------------------------------------------
template <int N>
struct Basis {
  float ar[N], dr[N], as[N], ds[N], at[N], dt[N];
};

// Where an element record lives: global memory (read-only path) or a warp's
// shared-memory staging slot. Offsets are in floats.
template <bool SM>
struct CoefRef;
template <>
struct CoefRef<false> {
  const float* __restrict__ p;
  __device__ __forceinline__ float4 ld4(int off) const { return __ldg(reinterpret_cast<const float4*>(p + off)); }
  __device__ __forceinline__ CoefRef at(int off) const { return CoefRef{p + off}; }
};
template <>
struct CoefRef<true> {
  uint32_t a;  // shared-space byte address
  __device__ __forceinline__ float4 ld4(int off) const {
    float4 v;
    asm("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a + 4u * off));
    return v;
  }
  __device__ __forceinline__ CoefRef at(int off) const { return CoefRef{a + 4u * static_cast<uint32_t>(off)}; }
};

// One coefficient row (N values) into registers, RS/4 vector loads.
template <int N, bool SM>
__device__ __forceinline__ void load_row(const CoefRef<SM>& c, int off, float (&r)[row_stride(N)]) {
#pragma unroll
  for (int q = 0; q < row_stride(N) / 4; ++q) {
    const float4 v = c.ld4(off + 4 * q);
    r[4 * q] = v.x;
    r[4 * q + 1] = v.y;
    r[4 * q + 2] = v.z;
    r[4 * q + 3] = v.w;
  }
}

// value and the three reference-space partials: out = {v, dv/dr, dv/ds, dv/dt}
template <int N, bool SM>
__device__ __noinline__ void contract_vd(CoefRef<SM> c, const Basis<N>* __restrict__ B, float* __restrict__ out) {
  constexpr int RS = row_stride(N);
  float ar[N], dr[N], as[N], ds[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    ar[i] = B->ar[i];
    dr[i] = B->dr[i];
    as[i] = B->as[i];
    ds[i] = B->ds[i];
  }
  float v = 0.f, vr = 0.f, vs = 0.f, vt = 0.f;
#pragma unroll 1
  for (int k = 0; k < N; ++k) {
    const float tk = B->at[k], dtk = B->dt[k];
    float q0 = 0.f, q1 = 0.f, q2 = 0.f;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      float row[RS];
      load_row<N, SM>(c, (k * N + j) * RS, row);
      float s0 = 0.f, s1 = 0.f;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        s0 = fmaf(row[i], ar[i], s0);
        s1 = fmaf(row[i], dr[i], s1);
      }
      q0 = fmaf(s0, as[j], q0);
      q1 = fmaf(s1, as[j], q1);
      q2 = fmaf(s0, ds[j], q2);
    }
    v = fmaf(q0, tk, v);
    vr = fmaf(q1, tk, vr);
    vs = fmaf(q2, tk, vs);
    vt = fmaf(q0, dtk, vt);
  }
  out[0] = v;
  out[1] = vr;
  out[2] = vs;
  out[3] = vt;
}

// value only
template <int N, bool SM>
__device__ __noinline__ float contract_v(CoefRef<SM> c, const Basis<N>* __restrict__ B) {
  constexpr int RS = row_stride(N);
  float ar[N], as[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    ar[i] = B->ar[i];
    as[i] = B->as[i];
  }
  float v = 0.0f;
#pragma unroll 1
  for (int k = 0; k < N; ++k) {
    const float tk = B->at[k];
    float q0 = 0.f;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      float row[RS];
      load_row<N, SM>(c, (k * N + j) * RS, row);
      float s0 = 0.f;
#pragma unroll
      for (int i = 0; i < N; ++i) s0 = fmaf(row[i], ar[i], s0);
      q0 = fmaf(s0, as[j], q0);
    }
    v = fmaf(q0, tk, v);
  }
  return v;
}

// Element record (record_floats(N) floats): x, y, z geometry blocks then the
// field block, in global memory (SM = false) or a shared-memory slot.
template <int N, bool SM = false>
struct Elem {
  CoefRef<SM> c;
  bool has_field;
  __device__ __forceinline__ CoefRef<SM> fld() const { return c.at(3 * block_floats(N)); }
};

// x(xi) and J (row-major J[row=x,y,z][col=r,s,t]).
template <int N, bool SM>
__device__ __noinline__ void geom_eval_raw(CoefRef<SM> c, float3 xi, float* __restrict__ xJ) {
  Basis<N> B;
  basis_val_der<N>(xi.x, B.ar, B.dr);
  basis_val_der<N>(xi.y, B.as, B.ds);
  basis_val_der<N>(xi.z, B.at, B.dt);
#pragma unroll 1
  for (int comp = 0; comp < 3; ++comp) contract_vd<N, SM>(c.at(comp * block_floats(N)), &B, xJ + 4 * comp);
}

template <int N, bool SM>
__device__ __forceinline__ void geom_eval(const Elem<N, SM>& e, float3 xi, float3& x, float (&J)[9], Work& w) {
  float r[12];
  geom_eval_raw<N, SM>(e.c, xi, r);
  x = make_float3(r[0], r[4], r[8]);
  J[0] = r[1]; J[1] = r[2]; J[2] = r[3];
  J[3] = r[5]; J[4] = r[6]; J[5] = r[7];
  J[6] = r[9]; J[7] = r[10]; J[8] = r[11];
  ++w.geom;
}

template <int N, bool SM>
__device__ __noinline__ float3 geom_map_raw(CoefRef<SM> c, float3 xi) {
  Basis<N> B;
  basis_val<N>(xi.x, B.ar);
  basis_val<N>(xi.y, B.as);
  basis_val<N>(xi.z, B.at);
  const float x = contract_v<N, SM>(c, &B);
  const float y = contract_v<N, SM>(c.at(block_floats(N)), &B);
  const float z = contract_v<N, SM>(c.at(2 * block_floats(N)), &B);
  return make_float3(x, y, z);
}

template <int N, bool SM>
__device__ __forceinline__ float3 geom_map(const Elem<N, SM>& e, float3 xi, Work& w) {
  ++w.map;
  return geom_map_raw<N, SM>(e.c, xi);
}

// u(xi) and grad_xi u
template <int N, bool SM>
__device__ __noinline__ void field_eval_raw(CoefRef<SM> c, float3 xi, float* __restrict__ ug) {
  Basis<N> B;
  basis_val_der<N>(xi.x, B.ar, B.dr);
  basis_val_der<N>(xi.y, B.as, B.ds);
  basis_val_der<N>(xi.z, B.at, B.dt);
  contract_vd<N, SM>(c, &B, ug);
}

template <int N, bool SM>
__device__ __forceinline__ void field_eval(const Elem<N, SM>& e, float3 xi, float& u, float3& g, Work& w) {
  float r[4];
  field_eval_raw<N, SM>(e.fld(), xi, r);
  u = r[0];
  g = make_float3(r[1], r[2], r[3]);
  ++w.field;
}

template <int N, bool SM>
__device__ __noinline__ float field_value_raw(CoefRef<SM> c, float3 xi) {
  Basis<N> B;
  basis_val<N>(xi.x, B.ar);
  basis_val<N>(xi.y, B.as);
  basis_val<N>(xi.z, B.at);
  return contract_v<N, SM>(c, &B);
}

template <int N, bool SM>
__device__ __forceinline__ float field_value(const Elem<N, SM>& e, float3 xi) {
  return field_value_raw<N, SM>(e.fld(), xi);
}

// Components [c0, c1) of one point evaluation, out of line: 0-2 are x, y, z
// (value and the three partials), 3 is the field. The basis values stay in
// registers: the rolled k loop picks at[k] / dt[k] with a predicated select
// instead of reading them back from the stack, and one loop body serves all
// components, so the code stays small. Same FMA order as contract_vd.
template <int N, bool SM>
__device__ __noinline__ void eval_comps(CoefRef<SM> c, float3 xi, int c0, int c1, float4* __restrict__ out) {
  constexpr int RS = row_stride(N);
  float ar[N], dr[N], as[N], ds[N], at[N], dt[N];
  basis_val_der<N>(xi.x, ar, dr);
  basis_val_der<N>(xi.y, as, ds);
  basis_val_der<N>(xi.z, at, dt);
#pragma unroll 1
  for (int comp = c0; comp < c1; ++comp) {
    const CoefRef<SM> cc = c.at(comp * block_floats(N));
    float v = 0.f, vr = 0.f, vs = 0.f, vt = 0.f;
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
      float tk = at[0], dtk = dt[0];
#pragma unroll
      for (int m = 1; m < N; ++m)
        if (k == m) {
          tk = at[m];
          dtk = dt[m];
        }
      float q0 = 0.f, q1 = 0.f, q2 = 0.f;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        float row[RS];
        load_row<N, SM>(cc, (k * N + j) * RS, row);
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          s0 = fmaf(row[i], ar[i], s0);
          s1 = fmaf(row[i], dr[i], s1);
        }
        q0 = fmaf(s0, as[j], q0);
        q1 = fmaf(s1, as[j], q1);
        q2 = fmaf(s0, ds[j], q2);
      }
      v = fmaf(q0, tk, v);
      vr = fmaf(q1, tk, vr);
      vs = fmaf(q2, tk, vs);
      vt = fmaf(q0, dtk, vt);
    }
    out[comp] = make_float4(v, vr, vs, vt);
  }
}

// Adjugate / determinant inverse, no singular guard (HexElement.cu:208-225).
__device__ __forceinline__ void invert3(const float (&J)[9], float (&K)[9]) {
  const float c0 = J[4] * J[8] - J[5] * J[7];
  const float c1 = J[5] * J[6] - J[3] * J[8];
  const float c2 = J[3] * J[7] - J[4] * J[6];
  const float det = J[0] * c0 + J[1] * c1 + J[2] * c2;
  const float id = 1.0f / det;
  K[0] = c0 * id;
  K[1] = (J[2] * J[7] - J[1] * J[8]) * id;
  K[2] = (J[1] * J[5] - J[2] * J[4]) * id;
  K[3] = c1 * id;
  K[4] = (J[0] * J[8] - J[2] * J[6]) * id;
  K[5] = (J[2] * J[3] - J[0] * J[5]) * id;
  K[6] = c2 * id;
  K[7] = (J[1] * J[6] - J[0] * J[7]) * id;
  K[8] = (J[0] * J[4] - J[1] * J[3]) * id;
}

// Inverse map x(xi) = p by Newton from xi0 (the reference always starts at
// 0), at most 50 iterations, converged when every |delta| < 1e-5.
// A NaN iterate can never converge, so it stops early with the same answer.
template <int N, bool SM>
__device__ __forceinline__ bool inverse_map(const Elem<N, SM>& e, float3 p, float3& xi, Work& w,
                                            float3 xi0 = make_float3(0.f, 0.f, 0.f), int max_it = 50) {
  xi = xi0;
  for (int it = 0; it < max_it; ++it) {
    ++w.newton;
    float3 x;
    float J[9], K[9];
    geom_eval<N>(e, xi, x, J, w);
    const float rx = x.x - p.x, ry = x.y - p.y, rz = x.z - p.z;
    invert3(J, K);
    const float d0 = K[0] * rx + K[1] * ry + K[2] * rz;
    const float d1 = K[3] * rx + K[4] * ry + K[5] * rz;
    const float d2 = K[6] * rx + K[7] * ry + K[8] * rz;
    xi.x -= d0;
    xi.y -= d1;
    xi.z -= d2;
    if (fabsf(d0) < 1e-5f && fabsf(d1) < 1e-5f && fabsf(d2) < 1e-5f) return true;
    if (!(fabsf(d0) + fabsf(d1) + fabsf(d2) < FLT_MAX)) return false;  // NaN / Inf
  }
  return false;
}

// f(t) = u(x(t)) - iso and df/dt with the world gradient
// (RayIsosurface.cu:44-65).
struct Sample {
  float3 xi;
  float f, df;
  float3 g;
};

// The batched engines' form of a sample (AH = true in sample_along): every
// Newton iteration also evaluates the field (value and xi-gradient) at its
// point, and when the step converges (all components below 1e-5) the sample
// is taken to first order at the converged point, u(xi - step) = u(xi) -
// grad u . step (error O(|step|^2), below 1e-9), with the gradient mapped by
// the iteration's inverse Jacobian. The reference evaluates the field and the
// Jacobian once more at the converged point (sample_along with AH = false);
// the round kernel and the warp-per-ray kernel both use this form, with the
// same arithmetic, so they give the same answers.
template <int N, bool SM>
__device__ __forceinline__ bool sample_ahead(const Elem<N, SM>& e, float3 o, float3 d, float t, float iso, Sample& s,
                                             Work& w, float3 xi0, int max_it) {
  float3 xi = xi0;
  for (int it = 1;; ++it) {
    float4 r[4];
    eval_comps<N, SM>(e.c, xi, 0, 4, r);
    w.flops += eval_flops(N, 4);
    ++w.geom;
    ++w.field;
    const float J[9] = {r[0].y, r[0].z, r[0].w, r[1].y, r[1].z, r[1].w, r[2].y, r[2].z, r[2].w};
    const float u = r[3].x;
    const float3 gr = make_float3(r[3].y, r[3].z, r[3].w);
    float K[9];
    invert3(J, K);
    ++w.newton;
    w.flops += kSolveFlops;
    const float rx = r[0].x - (o.x + t * d.x), ry = r[1].x - (o.y + t * d.y), rz = r[2].x - (o.z + t * d.z);
    const float d0 = K[0] * rx + K[1] * ry + K[2] * rz;
    const float d1 = K[3] * rx + K[4] * ry + K[5] * rz;
    const float d2 = K[6] * rx + K[7] * ry + K[8] * rz;
    xi.x -= d0;
    xi.y -= d1;
    xi.z -= d2;
    if (fabsf(d0) < 1e-5f && fabsf(d1) < 1e-5f && fabsf(d2) < 1e-5f) {
      s.xi = xi;
      s.g = make_float3(K[0] * gr.x + K[3] * gr.y + K[6] * gr.z, K[1] * gr.x + K[4] * gr.y + K[7] * gr.z,
                        K[2] * gr.x + K[5] * gr.y + K[8] * gr.z);
      s.f = (u - (gr.x * d0 + gr.y * d1 + gr.z * d2)) - iso;
      s.df = s.g.x * d.x + s.g.y * d.y + s.g.z * d.z;
      return true;
    }
    s.xi = xi;
    if (!(fabsf(d0) + fabsf(d1) + fabsf(d2) < FLT_MAX)) return false;
    if (it >= max_it) return false;
  }
}

template <int N, bool SM, bool AH = false>
__device__ __forceinline__ bool sample_along(const Elem<N, SM>& e, float3 o, float3 d, float t, float iso, Sample& s,
                                             Work& w, float3 xi0 = make_float3(0.f, 0.f, 0.f), int max_it = 50) {
  if constexpr (AH) return sample_ahead<N, SM>(e, o, d, t, iso, s, w, xi0, max_it);
  const float3 p = make_float3(o.x + t * d.x, o.y + t * d.y, o.z + t * d.z);
  if (!inverse_map<N>(e, p, s.xi, w, xi0, max_it)) return false;
  float u;
  float3 gr;
  field_eval<N>(e, s.xi, u, gr, w);
  float3 x;
  float J[9], K[9];
  geom_eval<N>(e, s.xi, x, J, w);
  invert3(J, K);
  s.g = make_float3(K[0] * gr.x + K[3] * gr.y + K[6] * gr.z, K[1] * gr.x + K[4] * gr.y + K[7] * gr.z,
                    K[2] * gr.x + K[5] * gr.y + K[8] * gr.z);
  s.f = u - iso;
  s.df = s.g.x * d.x + s.g.y * d.y + s.g.z * d.z;
  return true;
}

// Learned-mode sample: Newton from a predicted xi with a short iteration cap;
// if that does not converge the plain cold-start solve answers (the fallback
// the learned guess never replaces).
constexpr int kWarmCap = 4;
template <int N, bool SM, bool AH = false>
__device__ __forceinline__ bool sample_warm(const Elem<N, SM>& e, float3 o, float3 d, float t, float iso, Sample& s,
                                            Work& w, bool warm, float3 xi0) {
  if (warm) {
    if (sample_along<N, SM, AH>(e, o, d, t, iso, s, w, xi0, kWarmCap)) {
      ++w.accepted;
      return true;
    }
    ++w.rejected;
  }
  return sample_along<N, SM, AH>(e, o, d, t, iso, s, w);
}

__device__ __forceinline__ float3 lerp3(float3 a, float3 b, float u) {
  return make_float3(a.x + u * (b.x - a.x), a.y + u * (b.y - a.y), a.z + u * (b.z - a.z));
}

// At most 20 safeguarded Newton/bisection steps on a bracket [lt, rt] whose
// left sample is ls; done when |f| < 1e-5, else the midpoint with the left
// sample's xi and gradient (RayIsosurface.cu:121-177).
template <int N, bool SM, bool AH = false>
__device__ __forceinline__ bool refine_bracket(const Elem<N, SM>& e, float3 o, float3 d, float iso, float lt, float rt,
                                               Sample ls, float& th, float3& xh, float3& gh, Work& w,
                                               bool warm = false, float3 rxi = make_float3(0.f, 0.f, 0.f)) {
  for (int it = 0; it < 20; ++it) {
    const float mt = 0.5f * (lt + rt);
    Sample ms;
    if (!sample_warm<N, SM, AH>(e, o, d, mt, iso, ms, w, warm, lerp3(ls.xi, rxi, 0.5f))) return false;
    float ct = mt;
    if (fabsf(ms.df) > 1e-8f) {
      const float nt = mt - ms.f / ms.df;
      if (nt > lt && nt < rt) ct = nt;
    }
    Sample cs;
    if (!sample_warm<N, SM, AH>(e, o, d, ct, iso, cs, w, warm, ms.xi)) {
      ct = mt;  // keep the failed solve's xi, as the reference does
      cs.f = ms.f;
      cs.g = ms.g;
    }
    if (fabsf(cs.f) < 1e-5f) {
      th = ct;
      xh = cs.xi;
      gh = cs.g;
      return true;
    }
    if (ls.f * cs.f <= 0.0f) {
      rt = ct;
      rxi = cs.xi;
    } else {
      lt = ct;
      ls = cs;
    }
  }
  th = 0.5f * (lt + rt);
  xh = ls.xi;
  gh = ls.g;
  return true;
}

// First sign change over 17 uniform samples of [t0,t1], then the bracket
// refinement (RayIsosurface.cu:67-188). One thread.
template <int N, bool SM>
__device__ bool find_iso(const Elem<N, SM>& e, float3 o, float3 d, float t0, float t1, float iso, float& th, float3& xh,
                         float3& gh, Work& w) {
  bool have = false;
  float tp = t0;
  Sample sp;
  sp.f = 0.f;
  sp.xi = make_float3(0.f, 0.f, 0.f);
  sp.g = sp.xi;
  for (int i = 0; i <= 16; ++i) {
    const float t = t0 + (t1 - t0) * (float(i) / 16.0f);
    Sample s;
    if (!sample_along<N>(e, o, d, t, iso, s, w)) continue;
    if (!have) {
      have = true;
      tp = t;
      sp = s;
      continue;
    }
    if (sp.f * s.f <= 0.0f) return refine_bracket<N>(e, o, d, iso, tp, t, sp, th, xh, gh, w);
    tp = t;
    sp = s;
  }
  return false;
}

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float3 shfl3(float3 v, int src) {
  return make_float3(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src), __shfl_sync(kFull, v.z, src));
}

// Warp version: the 17 samples are independent inverse-map solves, so lane i
// solves sample i; the first sample i (in order) that succeeded and whose
// previous successful sample has f(prev)*f(i) <= 0 is found with ballots —
// the same bracket the sequential scan stops at. The refinement is then run
// by every lane on identical data (uniform control flow); its work is
// counted in wu, which only lane 0 reports. Call with all 32 lanes. The
// samples take the field with every Newton iteration (sample_ahead), as the
// round kernel does.
// Learned prediction for one candidate: xi at the segment entry te and
// d xi / d t there (scaled by the element size: xi(t) ~ xi_in + (t-te)*k*v).
struct Pred {
  bool on;
  float3 xi_in, v;
  float k, te;
  __device__ __forceinline__ float3 at(float t) const {
    const float u = (t - te) * k;
    return make_float3(xi_in.x + u * v.x, xi_in.y + u * v.y, xi_in.z + u * v.z);
  }
};

template <int N, bool L, bool SM>
__device__ bool find_iso_warp(const Elem<N, SM>& e, float3 o, float3 d, float t0, float t1, float iso, float& th,
                              float3& xh, float3& gh, Work& w, Work& wu, const Pred& pr) {
  const int lane = threadIdx.x & 31;
  Sample s;
  s.f = 0.f;
  s.df = 0.f;
  s.xi = make_float3(0.f, 0.f, 0.f);
  s.g = s.xi;
  const long long c0 = clock64();
  const float t = t0 + (t1 - t0) * (float(lane) / 16.0f);
  bool ok = false;
  if (!L || !pr.on) {
    if (lane <= 16) ok = sample_along<N, SM, true>(e, o, d, t, iso, s, w);
  } else {
    // learned: Newton from the predicted xi, short cap
    if (lane <= 16) ok = sample_along<N, SM, true>(e, o, d, t, iso, s, w, pr.at(t), kWarmCap);
    // a sample that missed the cap restarts from its converged neighbours'
    // xi (interpolated in t), then, failing that, from the plain cold start
    const unsigned cm = __ballot_sync(kFull, ok && lane <= 16);
    const unsigned lt_mask = (1u << lane) - 1u;
    const unsigned below = cm & lt_mask, above = cm & ~lt_mask & ~(1u << lane) & 0x1FFFFu;
    const int lb = below ? 31 - __clz(below) : lane, la = above ? __ffs(above) - 1 : lane;
    const float3 xb = shfl3(s.xi, lb), xa = shfl3(s.xi, la);
    const float tb = __shfl_sync(kFull, t, lb), ta = __shfl_sync(kFull, t, la);
    if (lane <= 16) {
      if (ok) {
        ++w.accepted;
      } else {
        float3 g0 = pr.at(t);
        if (below && above) g0 = lerp3(xb, xa, (t - tb) / (ta - tb));
        else if (below) g0 = make_float3(xb.x + (t - tb) * pr.k * pr.v.x, xb.y + (t - tb) * pr.k * pr.v.y,
                                         xb.z + (t - tb) * pr.k * pr.v.z);
        else if (above) g0 = make_float3(xa.x + (t - ta) * pr.k * pr.v.x, xa.y + (t - ta) * pr.k * pr.v.y,
                                         xa.z + (t - ta) * pr.k * pr.v.z);
        ok = (cm != 0u) && sample_along<N, SM, true>(e, o, d, t, iso, s, w, g0, kWarmCap);
        if (!ok) {
          ++w.rejected;
          ok = sample_along<N, SM, true>(e, o, d, t, iso, s, w);
        }
      }
    }
  }
  wu.cyc[1] += clock64() - c0;
  const unsigned okm = __ballot_sync(kFull, ok);
  const unsigned below = okm & ((1u << lane) - 1u);
  const int prev = below ? 31 - __clz(below) : lane;
  const float pf = __shfl_sync(kFull, s.f, prev);
  const bool sc = ok && below != 0u && pf * s.f <= 0.0f;
  const unsigned scm = __ballot_sync(kFull, sc);
  if (scm == 0u) return false;
  const int ri = __ffs(scm) - 1;
  const int li = 31 - __clz(okm & ((1u << ri) - 1u));
  const float lt = __shfl_sync(kFull, t, li), rt = __shfl_sync(kFull, t, ri);
  Sample ls;
  ls.f = __shfl_sync(kFull, s.f, li);
  ls.df = __shfl_sync(kFull, s.df, li);
  ls.xi = shfl3(s.xi, li);
  ls.g = shfl3(s.g, li);
  const float3 rxi = shfl3(s.xi, ri);
  const long long c1 = clock64();
  const bool found = refine_bracket<N, SM, true>(e, o, d, iso, lt, rt, ls, th, xh, gh, wu, L && pr.on, rxi);
  wu.cyc[2] += clock64() - c1;
  return found;
}

// Slab test clipped to [tmin, tmax] (high_order.h:115-152).
__device__ __forceinline__ bool ray_box(float3 o, float3 d, const float* lo, const float* hi, float tmin, float tmax,
                                        float& te, float& tx) {
  te = tmin;
  tx = tmax;
  const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (fabsf(dd[a]) < 1e-8f) {
      if (oo[a] < lo[a] || oo[a] > hi[a]) return false;
      continue;
    }
    const float inv = 1.0f / dd[a];
    float a0 = (lo[a] - oo[a]) * inv, a1 = (hi[a] - oo[a]) * inv;
    if (a0 > a1) {
      const float tmp = a0;
      a0 = a1;
      a1 = tmp;
    }
    te = fmaxf(te, a0);
    tx = fminf(tx, a1);
  }
  return tx >= te;
}

// Face table (high_order.h:164-184): fixed axis, fixed value, free axes.
__device__ __forceinline__ void face_param(int f, int& fixed, float& val, int& ua, int& va) {
  switch (f) {
    case 0: fixed = 2; val = -1.f; ua = 0; va = 1; break;
    case 1: fixed = 1; val = -1.f; ua = 0; va = 2; break;
    case 2: fixed = 0; val = 1.f; ua = 1; va = 2; break;
    case 3: fixed = 1; val = 1.f; ua = 0; va = 2; break;
    case 4: fixed = 0; val = -1.f; ua = 1; va = 2; break;
    default: fixed = 2; val = 1.f; ua = 0; va = 1; break;
  }
}

__device__ __forceinline__ float getc(float3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ void setc(float3& v, int a, float s) {
  if (a == 0) v.x = s;
  else if (a == 1) v.y = s;
  else v.z = s;
}

// One seed of the ray / curved-face Newton in (u,v,tau): at most 50
// iterations, accept when max|X-Y| < 1e-4 with u,v in [-1.001,1.001] and tau
// in [tmin,tmax]; step clamp 0.25, divergence break after 5 iterations
// (high_order.h:213-300).
template <int N, bool SM>
__device__ bool face_newton(const Elem<N, SM>& e, float3 o, float3 d, int f, float3 p, float tau, float tmin, float tmax,
                            float& th, float3& xh, Work& w, int max_it);

template <int N, bool SM>
__device__ bool face_seed(const Elem<N, SM>& e, float3 o, float3 d, int f, int si, int sj, float tmin, float tmax,
                          float& th, float3& xh, Work& w) {
  int fixed, ua, va;
  float val;
  face_param(f, fixed, val, ua, va);
  const float dd = d.x * d.x + d.y * d.y + d.z * d.z;
  float3 p = make_float3(0.f, 0.f, 0.f);
  setc(p, fixed, val);
  setc(p, ua, si == 0 ? -0.8f : (si == 1 ? 0.0f : 0.8f));
  setc(p, va, sj == 0 ? -0.8f : (sj == 1 ? 0.0f : 0.8f));
  const float3 x0 = geom_map<N>(e, p, w);
  const float3 df = make_float3(x0.x - o.x, x0.y - o.y, x0.z - o.z);
  float tau = dd > 0.f ? (df.x * d.x + df.y * d.y + df.z * d.z) / dd : 0.f;
  tau = fminf(fmaxf(tau, tmin), tmax);
  return face_newton<N>(e, o, d, f, p, tau, tmin, tmax, th, xh, w, 50);
}

// The (u,v,tau) Newton of one seed from a given start point.
template <int N, bool SM>
__device__ bool face_newton(const Elem<N, SM>& e, float3 o, float3 d, int f, float3 p, float tau, float tmin, float tmax,
                            float& th, float3& xh, Work& w, int max_it) {
  int fixed, ua, va;
  float val;
  face_param(f, fixed, val, ua, va);
  float prev = FLT_MAX;
  for (int it = 0; it < max_it; ++it) {
    ++w.face;
    float3 X;
    float J[9];
    geom_eval<N>(e, p, X, J, w);
    const float rx = X.x - (o.x + tau * d.x), ry = X.y - (o.y + tau * d.y), rz = X.z - (o.z + tau * d.z);
    const float m = fmaxf(fabsf(rx), fmaxf(fabsf(ry), fabsf(rz)));
    if (m < 1e-4f) {
      const float pu = getc(p, ua), pv = getc(p, va);
      if (pu >= -1.001f && pu <= 1.001f && pv >= -1.001f && pv <= 1.001f && tau >= tmin && tau <= tmax) {
        th = tau;
        xh = p;
        return true;
      }
      return false;
    }
    if (it > 5 && m > prev * 1.5f) return false;
    prev = m;
    const float A[9] = {J[ua], J[va], -d.x, J[3 + ua], J[3 + va], -d.y, J[6 + ua], J[6 + va], -d.z};
    float K[9];
    invert3(A, K);
    const float du = -(K[0] * rx + K[1] * ry + K[2] * rz);
    const float dv = -(K[3] * rx + K[4] * ry + K[5] * rz);
    const float dtau = -(K[6] * rx + K[7] * ry + K[8] * rz);
    const float mx = fmaxf(fabsf(du), fmaxf(fabsf(dv), fabsf(dtau)));
    const float sc = mx > 0.25f ? 0.25f / mx : 1.0f;
    float nu = getc(p, ua) + du * sc, nv = getc(p, va) + dv * sc;
    tau = fminf(fmaxf(tau + dtau * sc, tmin), tmax);
    nu = fminf(fmaxf(nu, -1.5f), 1.5f);  // fminf/fmaxf drop a NaN, as on the host
    nv = fminf(fmaxf(nv, -1.5f), 1.5f);
    setc(p, ua, nu);
    setc(p, va, nv);
    setc(p, fixed, val);
  }
  return false;
}

// Ray against one curved face: the 9 seeds {-0.8,0,0.8}^2 in order (v outer,
// u inner); the first seed accepted answers (high_order.h:189-304).
template <int N, bool SM>
__device__ bool hit_face(const Elem<N, SM>& e, float3 o, float3 d, int f, float tmin, float tmax, float& th, float3& xh,
                         Work& w) {
  for (int sj = 0; sj < 3; ++sj)
    for (int si = 0; si < 3; ++si)
      if (face_seed<N>(e, o, d, f, si, sj, tmin, tmax, th, xh, w)) return true;
  return false;
}

// Nearest boundary-face hit over the 6 faces. A face is skipped when the
// segment [tmin,tmax] misses that face's hull box: the box bounds the face
// over u,v in [-1.001,1.001] and is inflated past the 1e-4 acceptance
// tolerance plus rounding, so no seed could have been accepted there and the
// reference's answer for the face is "no hit" (exact culling).
// The reference's padded-box pre-test (high_order.h:420-431) is the same box
// the candidate was admitted with, so it always passes here.
template <int N, bool SM>
__device__ bool hit_hex(const Elem<N, SM>& e, const float* __restrict__ fbox, float3 o, float3 d, float tmin, float tmax,
                        float& th, float3& xh, int& face, Work& w) {
  bool any = false;
  float best = tmax;
  for (int f = 0; f < 6; ++f) {
    const float* b = fbox + 6 * f;
    const float lo[3] = {__ldg(b + 0), __ldg(b + 1), __ldg(b + 2)};
    const float hi[3] = {__ldg(b + 3), __ldg(b + 4), __ldg(b + 5)};
    float a0, a1;
    if (!ray_box(o, d, lo, hi, tmin, tmax, a0, a1)) {
      ++w.culled;
      continue;
    }
    float tf;
    float3 xf;
    if (hit_face<N>(e, o, d, f, tmin, tmax, tf, xf, w)) {
      if (tf > tmin && tf < best) {
        best = tf;
        xh = xf;
        face = f;
        any = true;
      }
    }
  }
  if (any) th = best;
  return any;
}

__device__ __forceinline__ float3 normalize3(float3 v) {
  const float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
  const float s = 1.0f / l;
  return make_float3(v.x * s, v.y * s, v.z * s);
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

struct HitState {
  float t;
  int elem, face, kind;
  float3 xi, n;
  float u;
  uint32_t flags;
};

// Two candidates' hits this close in t claim one surface point: a face shared
// by two elements, an edge of two faces, a root in the overlap of two padded
// boxes. The reference keeps whichever its visit order and FP32 rounding put
// first. A hit that displaces the best one by less than this keeps the
// displaced hit as the ray's tie partner, and the final FP64 check decides
// between the two (fp64_tie_rule).
constexpr float kTieT = 1e-4f;

// The best hit (t = best_t; a miss has FLT_MAX) is about to become a hit at
// t_new < best_t: keep the old one as the tie partner when it is within
// kTieT, else drop the partner (it lies behind the old best, so further than
// kTieT from the new hit too). Blind stores: no read of the partner.
__device__ __forceinline__ void note_tie(const HitState& best, float best_t, float t_new, HitState* tie) {
  if (!tie) return;
  if (best_t - t_new <= kTieT) *tie = best;
  else tie->kind = HO_HIT_MISS;
}

// Per-candidate policy of the reference's hex branch: iso search on the
// padded-box segment when enabled; if it finds nothing, nearest curved face.
template <int N, bool SM>
__device__ void visit_candidate(const Elem<N, SM>& e, const float* __restrict__ fbox, int eidx, float3 o, float3 d,
                                float te, float tx, float iso, bool iso_on, HitState& best, Work& w,
                                HitState* tie = nullptr) {
  ++w.cand;
  float th;
  float3 xi, g;
  if (iso_on && e.has_field && find_iso<N>(e, o, d, te, tx, iso, th, xi, g, w)) {
    if (th > 0.001f && th < best.t) {
      float3 n = normalize3(g);
      if (n.x * d.x + n.y * d.y + n.z * d.z > 0.f) n = make_float3(-n.x, -n.y, -n.z);
      note_tie(best, best.t, th, tie);
      best.t = th;
      best.elem = eidx;
      best.face = -1;
      best.kind = HO_HIT_ISO;
      best.xi = xi;
      best.n = n;
      best.u = field_value<N>(e, xi);
    }
    return;
  }
  int face = -1;
  if (hit_hex<N>(e, fbox, o, d, 0.001f, best.t, th, xi, face, w)) {
    if (th > 0.001f && th < best.t) {
      float3 x;
      float J[9];
      geom_eval<N>(e, xi, x, J, w);
      const float3 dr = make_float3(J[0], J[3], J[6]), ds = make_float3(J[1], J[4], J[7]),
                   dt = make_float3(J[2], J[5], J[8]);
      float3 n;
      if (fabsf(xi.x) > 0.9f) n = cross3(ds, dt);
      else if (fabsf(xi.y) > 0.9f) n = cross3(dr, dt);
      else n = cross3(dr, ds);
      n = normalize3(n);
      if (n.x * d.x + n.y * d.y + n.z * d.z > 0.f) n = make_float3(-n.x, -n.y, -n.z);
      note_tie(best, best.t, th, tie);
      best.t = th;
      best.elem = eidx;
      best.face = face;
      best.kind = HO_HIT_FACE;
      best.xi = xi;
      best.n = n;
      best.u = e.has_field ? field_value<N>(e, xi) : 0.f;
    }
  }
}

// Face test of one face against [tmin,tmax] through its hull box (exact cull).
__device__ __forceinline__ bool face_may_hit(const float* __restrict__ fbox, int f, float3 o, float3 d, float tmin,
                                             float tmax) {
  const float* b = fbox + 6 * f;
  const float lo[3] = {__ldg(b + 0), __ldg(b + 1), __ldg(b + 2)};
  const float hi[3] = {__ldg(b + 3), __ldg(b + 4), __ldg(b + 5)};
  float a0, a1;
  return ray_box(o, d, lo, hi, tmin, tmax, a0, a1);
}

// Warp version of hit_hex: the (face, seed) Newton solves of the faces that
// survive the cull are independent, so they are spread over the lanes (at
// most 6 x 9 = 54, two per lane). For each face the lowest seed index that
// was accepted answers — the seed the sequential loop would stop at — and
// faces are then compared in index order as the reference does.
// Where the predicted xi-line enters [-1,1]^3: face, start point, t.
__device__ __forceinline__ bool predicted_entry(const Pred& pr, float tmin, float tmax, int& face, float3& p,
                                                float& tau) {
  const float a[3] = {pr.xi_in.x, pr.xi_in.y, pr.xi_in.z};
  const float v[3] = {pr.v.x * pr.k, pr.v.y * pr.k, pr.v.z * pr.k};
  float enter = -FLT_MAX, leave = FLT_MAX;
  int ax = -1;
  float side = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (fabsf(v[c]) < 1e-12f) {
      if (fabsf(a[c]) > 1.f) return false;
      continue;
    }
    const float t0 = pr.te + (-1.f - a[c]) / v[c], t1 = pr.te + (1.f - a[c]) / v[c];
    const float lo = fminf(t0, t1), hi = fmaxf(t0, t1);
    if (lo > enter) {
      enter = lo;
      ax = c;
      side = (t0 < t1) ? -1.f : 1.f;
    }
    leave = fminf(leave, hi);
  }
  if (ax < 0 || enter > leave || enter > tmax || leave < tmin) return false;
  // face table (high_order.h:164-184): (axis, side) -> face index
  face = ax == 2 ? (side < 0.f ? 0 : 5) : (ax == 1 ? (side < 0.f ? 1 : 3) : (side < 0.f ? 4 : 2));
  tau = fminf(fmaxf(enter, tmin), tmax);
  p = pr.at(tau);
  setc(p, ax, side);
  return true;
}

template <int N, bool L, bool SM>
__device__ bool hit_hex_warp(const Elem<N, SM>& e, const float* __restrict__ fbox, float3 o, float3 d, float tmin,
                             float tmax, float& th, float3& xh, int& face, Work& w, Work& wu, const Pred& pr) {
  const int lane = threadIdx.x & 31;
  unsigned packed = 0;
  int na = 0;
  // learned: one Newton solve from the predicted element entry; faces whose
  // hull box misses [tmin, t_learned] cannot hold a nearer hit and are skipped
  int lf = -1;
  float lt = 0.f;
  float3 lx = make_float3(0.f, 0.f, 0.f);
  if (L && pr.on) {
    float3 p0;
    float tau0;
    int f0;
    if (predicted_entry(pr, tmin, tmax, f0, p0, tau0) &&
        face_newton<N>(e, o, d, f0, p0, tau0, tmin, tmax, lt, lx, wu, kWarmCap)) {
      lf = f0;
      ++wu.accepted;
    } else {
      ++wu.rejected;
    }
  }
  const float cull_hi = lf >= 0 ? lt : tmax;
  for (int f = 0; f < 6; ++f) {
    if (f != lf && face_may_hit(fbox, f, o, d, tmin, cull_hi)) {
      packed |= static_cast<unsigned>(f) << (3 * na);
      ++na;
    } else if (f != lf) {
      ++wu.culled;
    }
  }
  if (na == 0) {
    if (lf < 0 || !(lt > tmin && lt < tmax)) return false;
    th = lt;
    xh = lx;
    face = lf;
    return true;
  }
  const int T = na * 9;
  bool ok[2] = {false, false};
  float tv[2] = {0.f, 0.f};
  float3 xv[2] = {make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)};
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int k = lane + 32 * r;
    if (k < T) {
      const int slot = k / 9, sd = k - 9 * slot;
      const int f = (packed >> (3 * slot)) & 7u;
      ok[r] = face_seed<N>(e, o, d, f, sd % 3, sd / 3, tmin, tmax, tv[r], xv[r], w);
    }
  }
  bool any = false;
  float best = tmax;
  int a = 0;  // next surviving slot, in increasing face order
  for (int f = 0; f < 6; ++f) {
    float tf;
    float3 xf;
    if (f == lf) {
      tf = lt;
      xf = lx;
    } else {
      if (a >= na || static_cast<int>((packed >> (3 * a)) & 7u) != f) continue;
      const int k0 = lane, k1 = lane + 32;
      const unsigned b0 = __ballot_sync(kFull, ok[0] && k0 / 9 == a);
      const unsigned b1 = __ballot_sync(kFull, ok[1] && k1 < T && k1 / 9 == a);
      ++a;
      if ((b0 | b1) == 0u) continue;
      const bool second = b0 == 0u;
      const int src = second ? __ffs(b1) - 1 : __ffs(b0) - 1;
      const float tA = __shfl_sync(kFull, tv[0], src), tB = __shfl_sync(kFull, tv[1], src);
      const float3 xA = shfl3(xv[0], src), xB = shfl3(xv[1], src);
      tf = second ? tB : tA;
      xf = second ? xB : xA;
    }
    if (tf > tmin && tf < best) {
      best = tf;
      xh = xf;
      face = f;
      any = true;
    }
  }
  if (any) th = best;
  return any;
}

// Warp version of visit_candidate: every lane holds the same `best`.
template <int N, bool L, bool SM>
__device__ void visit_warp(const Elem<N, SM>& e, const float* __restrict__ fbox, int eidx, float3 o, float3 d, float te,
                           float tx, float iso, bool iso_on, HitState& best, Work& w, Work& wu, const Pred& pr,
                           HitState* tie = nullptr) {
  ++wu.cand;
  float th;
  float3 xi, g;
  if (iso_on && e.has_field && find_iso_warp<N, L>(e, o, d, te, tx, iso, th, xi, g, w, wu, pr)) {
    if (th > 0.001f && th < best.t) {
      float3 n = normalize3(g);
      if (n.x * d.x + n.y * d.y + n.z * d.z > 0.f) n = make_float3(-n.x, -n.y, -n.z);
      note_tie(best, best.t, th, tie);
      best.t = th;
      best.elem = eidx;
      best.face = -1;
      best.kind = HO_HIT_ISO;
      best.xi = xi;
      best.n = n;
      float4 r[4];  // the field at the root, as the round kernel's post evaluation
      eval_comps<N, SM>(e.c, xi, 3, 4, r);
      best.u = r[3].x;
    }
    return;
  }
  int face = -1;
  const long long c0 = clock64();
  const bool fh = hit_hex_warp<N, L>(e, fbox, o, d, 0.001f, best.t, th, xi, face, w, wu, pr);
  wu.cyc[3] += clock64() - c0;
  if (fh) {
    if (th > 0.001f && th < best.t) {
      // geometry (and field) at the hit, as the round kernel's post evaluation
      float4 r[4];
      eval_comps<N, SM>(e.c, xi, 0, e.has_field ? 4 : 3, r);
      ++wu.geom;
      const float3 dr = make_float3(r[0].y, r[1].y, r[2].y), ds = make_float3(r[0].z, r[1].z, r[2].z),
                   dt = make_float3(r[0].w, r[1].w, r[2].w);
      float3 n;
      if (fabsf(xi.x) > 0.9f) n = cross3(ds, dt);
      else if (fabsf(xi.y) > 0.9f) n = cross3(dr, dt);
      else n = cross3(dr, ds);
      n = normalize3(n);
      if (n.x * d.x + n.y * d.y + n.z * d.z > 0.f) n = make_float3(-n.x, -n.y, -n.z);
      note_tie(best, best.t, th, tie);
      best.t = th;
      best.elem = eidx;
      best.face = face;
      best.kind = HO_HIT_FACE;
      best.xi = xi;
      best.n = n;
      best.u = e.has_field ? r[3].x : 0.f;
    }
  }
}

}  // namespace ho
