// Final FP64 residual check of every hit and the plain-solver fallback for
// the hits that fail it (batched and learned modes).
//
// The FP32 solves stop on the reference's own criteria (inverse-map step
// below 1e-5, surface residual below 1e-4, isosurface |f| below 1e-5). The
// check re-evaluates the returned point in FP64 from the element's
// coefficients: the position x(xi) against o + t d, and for an isosurface
// hit the field u(xi) against the isovalue. A hit that fails is traced again
// by the plain cold-start solver (the reference's per-ray structure), whose
// answer replaces it; if that answer fails too it is kept and flagged
// HO_FLAG_FP64_FAIL.
#pragma once

#include <cuda_runtime.h>

#include "ho_rounds.cuh"
#include "ho_trace.cuh"

namespace ho {

// Tolerances of the check, FP64 and absolute (the scene is O(1)): the face
// acceptance 1e-4 and the isosurface criterion 1e-5, each with room for the
// FP32 rounding of the returned point.
constexpr double kCheckFaceTol = 1.5e-4;
constexpr double kCheckIsoPosTol = 1e-4;
constexpr double kCheckIsoFieldTol = 2e-5;

// Modified-A basis values in FP64, the recurrence of basis_val.
template <int N>
__device__ __forceinline__ void basis_val64(double x, double (&a)[N]) {
  a[0] = 0.5 * (1.0 - x);
  if (N > 1) a[1] = 0.5 * (1.0 + x);
  const double w = 0.25 * (1.0 - x * x);
  double pm2 = 1.0, pm1 = 2.0 * x;
#pragma unroll
  for (int i = 2; i < N; ++i) {
    const int m = i - 2;
    double p;
    if (m == 0) p = 1.0;
    else if (m == 1) p = pm1;
    else {
      const double A = double((2 * m + 1) * (m + 1)) / double(m * (m + 2));
      const double B = double(m + 1) / double(m + 2);
      p = A * x * pm1 - B * pm2;
      pm2 = pm1;
      pm1 = p;
    }
    a[i] = w * p;
  }
}

// Knuth's TwoSum: s + e == a + b exactly (round-to-nearest FP32; the
// intrinsics keep the compiler from fusing or reordering the steps).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Value of one coefficient block (rows padded to row_stride(N), a multiple of
// 4 floats, so a row is RS/4 aligned float4 loads), FP64-accurate.
//
// The coefficients are FP32, so the innermost sums sum_i c_i a_i are formed
// in double-single arithmetic on the FP32 pipes: a_i = ah_i + al_i (two
// floats), c_i ah_i = p + ep exactly (FMA-based TwoProduct), the running sum
// kept as sh + sl with TwoSum, the small parts added in FP32. That is about
// 2^-44 relative per row, below FP64's own rounding of the outer sums, and
// avoids an FP64 conversion and FMA per coefficient (FP64 runs at a small
// fraction of the FP32 rate here). The sums over j and k, and the residuals,
// are FP64.
template <int N>
__device__ double value64(const float* __restrict__ blk, const float (&ah)[N], const float (&al)[N],
                          const double (&as)[N], const double (&at)[N]) {
  constexpr int RS = row_stride(N);
  static_assert(RS % 4 == 0, "rows are whole float4s");
  double v = 0.0;
#pragma unroll 1
  for (int k = 0; k < N; ++k) {
    double q = 0.0;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const float4* row = reinterpret_cast<const float4*>(blk + (k * N + j) * RS);
      float c[RS];
#pragma unroll
      for (int i4 = 0; i4 < RS / 4; ++i4) {
        const float4 t4 = __ldg(row + i4);
        c[4 * i4] = t4.x;
        c[4 * i4 + 1] = t4.y;
        c[4 * i4 + 2] = t4.z;
        c[4 * i4 + 3] = t4.w;
      }
      float sh = 0.f, sl = 0.f;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const float p = __fmul_rn(c[i], ah[i]);
        const float ep = __fmaf_rn(c[i], ah[i], -p);
        float s, es;
        two_sum(sh, p, s, es);
        sh = s;
        sl = __fadd_rn(sl, __fadd_rn(__fadd_rn(es, ep), __fmul_rn(c[i], al[i])));
      }
      q = fma(static_cast<double>(sh) + static_cast<double>(sl), as[j], q);
    }
    double atk = 0.0;  // at[k] by selection: the array stays in registers
#pragma unroll
    for (int kk = 0; kk < N; ++kk)
      if (kk == k) atk = at[kk];
    v = fma(q, atk, v);
  }
  return v;
}

// The FP64 residuals of a hit at xi in element elem: the largest component
// of x(xi) - (o + t d), and the field value u(xi) (0 when unused).
template <int N>
__device__ void fp64_residuals(const float* __restrict__ rec_all, int elem, float3 o, float3 d, float t, float3 xi,
                               bool want_field, double& rpos, double& u) {
  const float* rec = rec_all + static_cast<int64_t>(elem) * record_floats(N);
  double ar[N], as[N], at[N];
  basis_val64<N>(static_cast<double>(xi.x), ar);
  basis_val64<N>(static_cast<double>(xi.y), as);
  basis_val64<N>(static_cast<double>(xi.z), at);
  float ah[N], al[N];  // ar as two floats
#pragma unroll
  for (int i = 0; i < N; ++i) {
    ah[i] = static_cast<float>(ar[i]);
    al[i] = static_cast<float>(ar[i] - static_cast<double>(ah[i]));
  }
  const double td = t;
  const double px = static_cast<double>(o.x) + td * d.x, py = static_cast<double>(o.y) + td * d.y,
               pz = static_cast<double>(o.z) + td * d.z;
  const double rx = fabs(value64<N>(rec, ah, al, as, at) - px);
  const double ry = fabs(value64<N>(rec + block_floats(N), ah, al, as, at) - py);
  const double rz = fabs(value64<N>(rec + 2 * block_floats(N), ah, al, as, at) - pz);
  rpos = fmax(rx, fmax(ry, rz));
  u = want_field ? value64<N>(rec + 3 * block_floats(N), ah, al, as, at) : 0.0;
}

// True when the hit passes the FP64 check (a miss always passes).
template <int N>
__device__ bool fp64_check(const TraceParams& P, float3 o, float3 d, float iso, const HitState& h) {
  if (h.kind == HO_HIT_MISS) return true;
  const bool iso_hit = h.kind != HO_HIT_FACE;
  double r, u;
  fp64_residuals<N>(P.rec, h.elem, o, d, h.t, h.xi, iso_hit, r, u);
  if (!iso_hit) return r <= kCheckFaceTol;
  if (r > kCheckIsoPosTol) return false;
  return fabs(u - static_cast<double>(iso)) <= kCheckIsoFieldTol;
}

// The check's residuals for given hits (ho_hit_residuals): per hit the
// position residual and the field value at its xi.
template <int N>
__global__ void __launch_bounds__(128) residual_kernel(const float* __restrict__ rec, const uint32_t* __restrict__ flags,
                                                       int64_t n, const float* __restrict__ rays,
                                                       const ho_hit* __restrict__ hits, double* __restrict__ out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const ho_hit h = hits[i];
  double r = 0.0, u = 0.0;
  if ((h.kind == HO_HIT_FACE || h.kind == HO_HIT_ISO) && h.elem >= 0) {
    const float* ray = rays + 6 * i;
    fp64_residuals<N>(rec, h.elem, make_float3(ray[0], ray[1], ray[2]), make_float3(ray[3], ray[4], ray[5]), h.t,
                      make_float3(h.xi[0], h.xi[1], h.xi[2]), (flags[h.elem] & 1u) != 0, r, u);
  }
  out[2 * i] = r;
  out[2 * i + 1] = u;
}

template <int N>
cudaError_t launch_residuals_n(const float* rec, const uint32_t* flags, int64_t n, const float* rays, const ho_hit* hits,
                               double* out, cudaStream_t s) {
  if (n > 0) residual_kernel<N><<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(rec, flags, n, rays, hits, out);
  return cudaGetLastError();
}

// One thread per listed ray (the queued rays with a hit): FP64 check;
// failures are listed.
template <int N>
__global__ void __launch_bounds__(128) check_kernel(TraceParams P, RayState* __restrict__ st,
                                                    const uint32_t* __restrict__ list,
                                                    const unsigned* __restrict__ n_list,
                                                    uint32_t* __restrict__ fail_list, unsigned* __restrict__ n_fail) {
  const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
  bool checked = false, failed = false;
  if (k < *n_list) {
    const unsigned item = list[k];
    RayState& r = st[item];
    if (r.best.kind != HO_HIT_MISS) {
      float3 o, d;
      float iso;
      bool iso_on;
      query_ray(P, P.work[item], o, d, iso, iso_on);
      checked = true;
      failed = !fp64_check<N>(P, o, d, iso, r.best);
      if (failed) fail_list[atomicAdd(n_fail, 1u)] = item;
    }
  }
  const unsigned cm = __ballot_sync(0xffffffffu, checked), fm = __ballot_sync(0xffffffffu, failed);
  if ((threadIdx.x & 31) == 0) {
    if (cm) atomicAdd(&P.stats->c[ST_CHECKED], static_cast<unsigned long long>(__popc(cm)));
    if (fm) atomicAdd(&P.stats->c[ST_CHECK_FAIL], static_cast<unsigned long long>(__popc(fm)));
  }
}

// The failed rays, traced again by the plain cold-start solver (grid-stride
// over the device-side count); the plain answer replaces the fast one.
template <int N>
__global__ void __launch_bounds__(kTraceBlock) fallback_kernel(TraceParams P, RayState* __restrict__ st,
                                                               const uint32_t* __restrict__ fail_list,
                                                               const unsigned* __restrict__ n_fail) {
  const unsigned n = *n_fail;
  Work w;
  unsigned long long newton = 0, face = 0;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const unsigned item = fail_list[k];
    float3 o, d;
    float iso;
    bool iso_on;
    query_ray(P, P.work[item], o, d, iso, iso_on);
    HitState b = plain_trace<N>(P, o, d, iso, iso_on, w);
    b.flags |= HO_FLAG_FALLBACK | (st[item].best.flags & HO_FLAG_OVERFLOW);
    if (!fp64_check<N>(P, o, d, iso, b)) {
      b.flags |= HO_FLAG_FP64_FAIL;
      atomicAdd(&P.stats->c[ST_CHECK_FINAL], 1ull);
    }
    st[item].best = b;
    st[item].its += static_cast<int>(w.newton + w.face);
    newton += w.newton;
    face += w.face;
    w.newton = 0;
    w.face = 0;
  }
  if (newton) atomicAdd(&P.stats->c[ST_NEWTON], newton);
  if (face) atomicAdd(&P.stats->c[ST_FACE], face);
  if (w.geom) atomicAdd(&P.stats->c[ST_GEOM], static_cast<unsigned long long>(w.geom));
  if (w.field) atomicAdd(&P.stats->c[ST_FIELD], static_cast<unsigned long long>(w.field));
  if (w.map) atomicAdd(&P.stats->c[ST_MAP], static_cast<unsigned long long>(w.map));
}

template <int N>
cudaError_t launch_check_n(const TraceParams& P, RayState* st, const uint32_t* list, const unsigned* n_list,
                           uint32_t* fail_list, unsigned* n_fail, int64_t n_cap, int sms, cudaStream_t s) {
  check_kernel<N><<<static_cast<unsigned>((n_cap + 127) / 128), 128, 0, s>>>(P, st, list, n_list, fail_list, n_fail);
  fallback_kernel<N><<<sms * 2, kTraceBlock, 0, s>>>(P, st, fail_list, n_fail);
  return cudaGetLastError();
}

extern template cudaError_t launch_check_n<2>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<3>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<4>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<5>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<6>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<7>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<8>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<9>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, int64_t, int, cudaStream_t);

extern template cudaError_t launch_residuals_n<2>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);
extern template cudaError_t launch_residuals_n<3>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);
extern template cudaError_t launch_residuals_n<4>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);
extern template cudaError_t launch_residuals_n<5>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);
extern template cudaError_t launch_residuals_n<6>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);
extern template cudaError_t launch_residuals_n<7>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);
extern template cudaError_t launch_residuals_n<8>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);
extern template cudaError_t launch_residuals_n<9>(const float*, const uint32_t*, int64_t, const float*, const ho_hit*,
                                                  double*, cudaStream_t);

}  // namespace ho
