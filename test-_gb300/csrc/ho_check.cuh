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

// Value of one coefficient block (rows padded to row_stride(N), a multiple of
// 4 floats, so a row is RS/4 aligned float4 loads) in FP64. The rows of one k
// are independent and unrolled; each row sums even and odd terms separately
// to halve the dependent FMA chain.
template <int N>
__device__ double value64(const float* __restrict__ blk, const double (&ar)[N], const double (&as)[N],
                          const double (&at)[N]) {
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
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int i = 0; i < N; i += 2) s0 = fma(static_cast<double>(c[i]), ar[i], s0);
#pragma unroll
      for (int i = 1; i < N; i += 2) s1 = fma(static_cast<double>(c[i]), ar[i], s1);
      q = fma(s0 + s1, as[j], q);
    }
    double atk = 0.0;  // at[k] by selection: the array stays in registers
#pragma unroll
    for (int kk = 0; kk < N; ++kk)
      if (kk == k) atk = at[kk];
    v = fma(q, atk, v);
  }
  return v;
}

// True when the hit passes the FP64 check (a miss always passes).
template <int N>
__device__ bool fp64_check(const TraceParams& P, float3 o, float3 d, float iso, const HitState& h) {
  if (h.kind == HO_HIT_MISS) return true;
  const float* rec = P.rec + static_cast<int64_t>(h.elem) * record_floats(N);
  double ar[N], as[N], at[N];
  basis_val64<N>(static_cast<double>(h.xi.x), ar);
  basis_val64<N>(static_cast<double>(h.xi.y), as);
  basis_val64<N>(static_cast<double>(h.xi.z), at);
  const double t = h.t;
  const double px = static_cast<double>(o.x) + t * d.x, py = static_cast<double>(o.y) + t * d.y,
               pz = static_cast<double>(o.z) + t * d.z;
  const double rx = fabs(value64<N>(rec, ar, as, at) - px);
  const double ry = fabs(value64<N>(rec + block_floats(N), ar, as, at) - py);
  const double rz = fabs(value64<N>(rec + 2 * block_floats(N), ar, as, at) - pz);
  const double r = fmax(rx, fmax(ry, rz));
  if (h.kind == HO_HIT_FACE) return r <= kCheckFaceTol;
  if (r > kCheckIsoPosTol) return false;
  const double u = value64<N>(rec + 3 * block_floats(N), ar, as, at);
  return fabs(u - static_cast<double>(iso)) <= kCheckIsoFieldTol;
}

// One thread per queued ray with a hit: FP64 check; failures are listed.
template <int N>
__global__ void __launch_bounds__(128) check_kernel(TraceParams P, RayState* __restrict__ st,
                                                    uint32_t* __restrict__ fail_list, unsigned* __restrict__ n_fail) {
  const unsigned item = blockIdx.x * blockDim.x + threadIdx.x;
  bool checked = false, failed = false;
  if (item < *P.qcount) {
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
cudaError_t launch_check_n(const TraceParams& P, RayState* st, uint32_t* fail_list, unsigned* n_fail, int64_t n_cap,
                           int sms, cudaStream_t s) {
  check_kernel<N><<<static_cast<unsigned>((n_cap + 127) / 128), 128, 0, s>>>(P, st, fail_list, n_fail);
  fallback_kernel<N><<<sms * 2, kTraceBlock, 0, s>>>(P, st, fail_list, n_fail);
  return cudaGetLastError();
}

extern template cudaError_t launch_check_n<2>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);
extern template cudaError_t launch_check_n<3>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);
extern template cudaError_t launch_check_n<4>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);
extern template cudaError_t launch_check_n<5>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);
extern template cudaError_t launch_check_n<6>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);
extern template cudaError_t launch_check_n<7>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);
extern template cudaError_t launch_check_n<8>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);
extern template cudaError_t launch_check_n<9>(const TraceParams&, RayState*, uint32_t*, unsigned*, int64_t, int,
                                              cudaStream_t);

}  // namespace ho
