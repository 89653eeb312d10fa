// Learned mode, data side: per-element descriptors (the geometric half of the
// network input) and training pairs produced by the plain solver.
//
// Descriptor of element e (48 floats): its 8 corners and 6 face-centre
// offsets (face centre minus the mean of that face's corners, x10) in the
// element's frame — centre c = mean of the corners, scale k = 1 / (largest
// extent of the corner box) — then c (3), k, and 2 zeros.
// Network input for a (ray, element) pair: descriptor[0:42], the ray's entry
// point into the element's padded box in the element frame, the unit ray
// direction: 48 values, BF16, zero-padded to 64.
// Targets: xi at that entry point (plain cold-start inverse map) and
// J(xi)^-1 d / k, the reference-space velocity per element-size unit of t.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "ho_device.cuh"
#include "ho_host.h"
#include "ho_learn.h"
#include "ho_mlp.h"

namespace ho {

template <int N>
__global__ void desc_kernel(const float* __restrict__ rec, int64_t n, float* __restrict__ desc) {
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float* r = rec + e * record_floats(N);
  Elem<N> el;
  el.c = CoefRef<false>{r};
  el.has_field = false;
  Work w;
  float cx[8][3];
  for (int v = 0; v < 8; ++v) {  // Z-order corner (i,j,k): vertex-mode coefficient
    const int i = v & 1, j = (v >> 1) & 1, k = v >> 2;
    for (int c = 0; c < 3; ++c) cx[v][c] = r[c * block_floats(N) + (k * N + j) * row_stride(N) + i];
  }
  float cen[3] = {0.f, 0.f, 0.f}, lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int v = 0; v < 8; ++v)
    for (int c = 0; c < 3; ++c) {
      cen[c] += 0.125f * cx[v][c];
      lo[c] = fminf(lo[c], cx[v][c]);
      hi[c] = fmaxf(hi[c], cx[v][c]);
    }
  const float ext = fmaxf(hi[0] - lo[0], fmaxf(hi[1] - lo[1], hi[2] - lo[2]));
  const float k = ext > 0.f ? 1.0f / ext : 1.0f;
  float* o = desc + e * kDescFloats;
  for (int v = 0; v < 8; ++v)
    for (int c = 0; c < 3; ++c) o[3 * v + c] = (cx[v][c] - cen[c]) * k;
  for (int f = 0; f < 6; ++f) {
    int fixed, ua, va;
    float val;
    face_param(f, fixed, val, ua, va);
    float3 p = make_float3(0.f, 0.f, 0.f);
    setc(p, fixed, val);
    const float3 x = geom_map<N>(el, p, w);
    float m[3] = {0.f, 0.f, 0.f};
    int cnt = 0;
    for (int v = 0; v < 8; ++v) {
      const int bit = (v >> fixed) & 1;
      if ((val < 0.f && bit == 0) || (val > 0.f && bit == 1)) {
        for (int c = 0; c < 3; ++c) m[c] += cx[v][c];
        ++cnt;
      }
    }
    const float xs[3] = {x.x, x.y, x.z};
    for (int c = 0; c < 3; ++c) o[24 + 3 * f + c] = 10.f * (xs[c] - m[c] / cnt) * k;
  }
  o[42] = cen[0];
  o[43] = cen[1];
  o[44] = cen[2];
  o[45] = k;
  o[46] = 0.f;
  o[47] = 0.f;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float unit_rand(uint64_t seed, uint64_t q, uint64_t k) {
  return static_cast<float>(mix64(seed ^ mix64(q * 16 + k)) >> 40) * (1.0f / 16777216.0f);
}

// One training pair per thread from the plain solver (cold-start inverse map).
template <int N>
__global__ void datagen_kernel(const float* __restrict__ rec, const float* __restrict__ box,
                               const float* __restrict__ desc, int64_t n_elem, int64_t n, uint64_t seed,
                               __nv_bfloat16* __restrict__ X, float* __restrict__ T, uint8_t* __restrict__ V) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int64_t e = static_cast<int64_t>(unit_rand(seed, q, 0) * n_elem) % n_elem;
  const float* b = box + 6 * e;
  const float3 p = make_float3(b[0] + unit_rand(seed, q, 1) * (b[3] - b[0]), b[1] + unit_rand(seed, q, 2) * (b[4] - b[1]),
                               b[2] + unit_rand(seed, q, 3) * (b[5] - b[2]));
  // uniform direction
  const float z = 2.f * unit_rand(seed, q, 4) - 1.f, ph = 6.28318530718f * unit_rand(seed, q, 5);
  const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
  const float3 d = make_float3(r * cosf(ph), r * sinf(ph), z);
  const float ext = fmaxf(b[3] - b[0], fmaxf(b[4] - b[1], b[5] - b[2]));
  const float3 o = make_float3(p.x - 2.f * ext * d.x, p.y - 2.f * ext * d.y, p.z - 2.f * ext * d.z);
  float te, tx;
  const float lo[3] = {b[0], b[1], b[2]}, hi[3] = {b[3], b[4], b[5]};
  bool ok = ray_box(o, d, lo, hi, 0.001f, FLT_MAX, te, tx);
  const float* ds = desc + e * kDescFloats;
  write_features(ds, o, d, ok ? te : 0.f, X + q * kMlpInPad);
  float* t = T + q * kMlpOut;
  for (int j = 0; j < kMlpOut; ++j) t[j] = 0.f;
  if (ok) {
    Elem<N> el;
    el.c = CoefRef<false>{rec + e * record_floats(N)};
    el.has_field = false;
    Work w;
    float3 xi;
    const float3 pin = make_float3(o.x + te * d.x, o.y + te * d.y, o.z + te * d.z);
    ok = inverse_map<N>(el, pin, xi, w);
    if (ok && fabsf(xi.x) < 3.f && fabsf(xi.y) < 3.f && fabsf(xi.z) < 3.f) {
      float3 x;
      float J[9], K[9];
      geom_eval<N>(el, xi, x, J, w);
      invert3(J, K);
      const float kk = ds[45];
      t[0] = xi.x;
      t[1] = xi.y;
      t[2] = xi.z;
      t[3] = (K[0] * d.x + K[1] * d.y + K[2] * d.z) / kk;
      t[4] = (K[3] * d.x + K[4] * d.y + K[5] * d.z) / kk;
      t[5] = (K[6] * d.x + K[7] * d.y + K[8] * d.z) / kk;
      ok = fabsf(t[3]) < 100.f && fabsf(t[4]) < 100.f && fabsf(t[5]) < 100.f;
    } else {
      ok = false;
    }
  }
  V[q] = ok ? 1 : 0;
}

#define DISPATCH_N(N_, CALL)                       \
  switch (N_) {                                    \
    case 2: { constexpr int NN = 2; CALL; } break; \
    case 3: { constexpr int NN = 3; CALL; } break; \
    case 4: { constexpr int NN = 4; CALL; } break; \
    case 5: { constexpr int NN = 5; CALL; } break; \
    case 6: { constexpr int NN = 6; CALL; } break; \
    case 7: { constexpr int NN = 7; CALL; } break; \
    case 8: { constexpr int NN = 8; CALL; } break; \
    case 9: { constexpr int NN = 9; CALL; } break; \
    default: return int(cudaErrorInvalidValue);    \
  }

int launch_desc(int N, const float* rec, int64_t n, float* desc, cudaStream_t s) {
  const unsigned blocks = static_cast<unsigned>((n + 127) / 128);
  DISPATCH_N(N, (desc_kernel<NN><<<blocks, 128, 0, s>>>(rec, n, desc)));
  return int(cudaGetLastError());
}

int launch_datagen(int N, const float* rec, const float* box, const float* desc, int64_t n_elem, int64_t n,
                   uint64_t seed, void* X, float* T, uint8_t* V, cudaStream_t s) {
  const unsigned blocks = static_cast<unsigned>((n + 127) / 128);
  DISPATCH_N(N, (datagen_kernel<NN><<<blocks, 128, 0, s>>>(rec, box, desc, n_elem, n, seed,
                                                           static_cast<__nv_bfloat16*>(X), T, V)));
  return int(cudaGetLastError());
}

}  // namespace ho
