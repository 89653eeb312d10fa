// Final FP64 residual check of every hit, the FP64 polish of the hits that
// pass it, and the plain-solver fallback for the hits that fail it.
//
// The FP32 solves stop on the reference's own criteria (inverse-map step
// below 1e-5, surface residual below 1e-4, isosurface |f| below 1e-5). The
// check re-evaluates the returned point in FP64 from the element's
// coefficients: the position x(xi) against o + t d, and for an isosurface
// hit the field u(xi) against the isovalue. A hit that fails is traced again
// by the plain cold-start solver (the reference's per-ray structure), whose
// answer replaces it; if that answer fails too it is kept and flagged
// HO_FLAG_FP64_FAIL. The check itself and the FP64 polish of the hits that
// pass it are in ho_fp64.cuh.
#pragma once

#include <cuda_runtime.h>

#include "ho_rounds.cuh"
#include "ho_trace.cuh"

namespace ho {

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

// One thread per listed ray (the queued rays with a hit): FP64 check and
// polish; failures are listed from the front of fail_list, rays that passed
// with a tie partner from its back (tie_end downwards: a listed ray goes to
// at most one of the two lists, so they do not meet).
template <int N>
__global__ void __launch_bounds__(128) check_kernel(TraceParams P, RayState* __restrict__ st,
                                                    const uint32_t* __restrict__ list,
                                                    const unsigned* __restrict__ n_list,
                                                    uint32_t* __restrict__ fail_list, unsigned* __restrict__ n_fail,
                                                    uint32_t* __restrict__ tie_end, unsigned* __restrict__ n_tie) {
  const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
  bool checked = false, failed = false, polished = false;
  if (k < *n_list) {
    const unsigned item = list[k];
    RayState& r = st[item];
    if (r.best.kind != HO_HIT_MISS) {
      float3 o, d;
      float iso;
      bool iso_on;
      query_ray(P, P.work[item], o, d, iso, iso_on);
      checked = true;
      HitState h = r.best;
      failed = !fp64_check_polish<N>(P.rec, P.flags, o, d, iso, h, polished);
      if (failed) {
        fail_list[atomicAdd(n_fail, 1u)] = item;
      } else {
        if (polished) r.best = h;
        if (r.tie.kind != HO_HIT_MISS) *(tie_end - atomicAdd(n_tie, 1u)) = item;
      }
    }
  }
  const unsigned cm = __ballot_sync(0xffffffffu, checked), fm = __ballot_sync(0xffffffffu, failed),
                 pm = __ballot_sync(0xffffffffu, polished);
  if ((threadIdx.x & 31) == 0) {
    if (cm) atomicAdd(&P.stats->c[ST_CHECKED], static_cast<unsigned long long>(__popc(cm)));
    if (fm) atomicAdd(&P.stats->c[ST_CHECK_FAIL], static_cast<unsigned long long>(__popc(fm)));
    if (pm) atomicAdd(&P.stats->c[ST_POLISHED], static_cast<unsigned long long>(__popc(pm)));
  }
}

// The rays the check listed with a tie partner, one thread each (grid-stride
// over the device-side count): the FP64 tie rule. A separate pass so that
// the partners, about 3% of the hits and spread over most warps, do not
// serialise the check's warps. The best hit is polished already; its exact
// root t is taken again by the same polish (one FP64 evaluation).
template <int N>
__global__ void __launch_bounds__(128) tie_kernel(TraceParams P, RayState* __restrict__ st,
                                                  const uint32_t* __restrict__ tie_end,
                                                  const unsigned* __restrict__ n_tie) {
  const unsigned n = *n_tie;
  unsigned long long weighed = 0, swapped = 0;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const unsigned item = *(tie_end - k);
    RayState& r = st[item];
    float3 o, d;
    float iso;
    bool iso_on;
    query_ray(P, P.work[item], o, d, iso, iso_on);
    HitState b = r.best;
    bool polished;
    double t64;
    if (!fp64_check_polish<N>(P.rec, P.flags, o, d, iso, b, polished, &t64)) continue;
    ++weighed;
    if (fp64_tie_rule<N>(P.rec, P.flags, o, d, iso, b, t64, r.tie)) ++swapped;
    r.best = b;
  }
  if (weighed) atomicAdd(&P.stats->c[ST_TIES], weighed);
  if (swapped) atomicAdd(&P.stats->c[ST_TIES_SWAPPED], swapped);
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
    HitState tie;
    HitState b = plain_trace<N>(P, o, d, iso, iso_on, w, &tie);
    b.flags |= HO_FLAG_FALLBACK | (st[item].best.flags & HO_FLAG_OVERFLOW);
    bool polished;
    double t64;
    if (!fp64_check_polish<N>(P.rec, P.flags, o, d, iso, b, polished, &t64)) {
      b.flags |= HO_FLAG_FP64_FAIL;
      atomicAdd(&P.stats->c[ST_CHECK_FINAL], 1ull);
    } else {
      if (polished) atomicAdd(&P.stats->c[ST_POLISHED], 1ull);
      if (tie.kind != HO_HIT_MISS) {
        atomicAdd(&P.stats->c[ST_TIES], 1ull);
        if (fp64_tie_rule<N>(P.rec, P.flags, o, d, iso, b, t64, tie)) atomicAdd(&P.stats->c[ST_TIES_SWAPPED], 1ull);
      }
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

// fail_list holds n_cap entries (n_cap >= the listed rays); n_fail and
// n_tie are zeroed by the caller.
template <int N>
cudaError_t launch_check_n(const TraceParams& P, RayState* st, const uint32_t* list, const unsigned* n_list,
                           uint32_t* fail_list, unsigned* n_fail, unsigned* n_tie, int64_t n_cap, int sms,
                           cudaStream_t s) {
  uint32_t* tie_end = fail_list + (n_cap - 1);
  check_kernel<N><<<static_cast<unsigned>((n_cap + 127) / 128), 128, 0, s>>>(P, st, list, n_list, fail_list, n_fail,
                                                                              tie_end, n_tie);
  tie_kernel<N><<<sms * 2, 128, 0, s>>>(P, st, tie_end, n_tie);
  fallback_kernel<N><<<sms * 2, kTraceBlock, 0, s>>>(P, st, fail_list, n_fail);
  return cudaGetLastError();
}

extern template cudaError_t launch_check_n<2>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<3>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<4>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<5>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<6>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<7>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<8>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);
extern template cudaError_t launch_check_n<9>(const TraceParams&, RayState*, const uint32_t*, const unsigned*,
                                              uint32_t*, unsigned*, unsigned*, int64_t, int, cudaStream_t);

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
