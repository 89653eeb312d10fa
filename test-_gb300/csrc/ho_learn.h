// Learned mode: element descriptors, network inputs, training-pair generation.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "ho_mlp.h"

namespace ho {

constexpr int kDescFloats = 48;  // see ho_learn.cu
constexpr int kPredK = 4;        // candidates per queued ray that get a prediction

// The ray-dependent inputs of a (ray, element) pair: the entry point in the
// element's frame (offset by the element's centre, scaled by its size) and
// the direction.
__device__ __forceinline__ void feature_tail(const float* __restrict__ desc, float3 o, float3 d, float te,
                                             float (&f)[6]) {
  const float k = desc[45];
  f[0] = (o.x + te * d.x - desc[42]) * k;
  f[1] = (o.y + te * d.y - desc[43]) * k;
  f[2] = (o.z + te * d.z - desc[44]) * k;
  f[3] = d.x;
  f[4] = d.y;
  f[5] = d.z;
}

// Network input of one (ray, element) pair, BF16 x 64 (48 used).
__device__ __forceinline__ void write_features(const float* __restrict__ desc, float3 o, float3 d, float te,
                                               __nv_bfloat16* __restrict__ row) {
  float f[6];
  feature_tail(desc, o, d, te, f);
  for (int j = 0; j < 42; j += 2)
    *reinterpret_cast<__nv_bfloat162*>(row + j) = __floats2bfloat162_rn(desc[j], desc[j + 1]);
  *reinterpret_cast<__nv_bfloat162*>(row + 42) = __floats2bfloat162_rn(f[0], f[1]);
  *reinterpret_cast<__nv_bfloat162*>(row + 44) = __floats2bfloat162_rn(f[2], f[3]);
  *reinterpret_cast<__nv_bfloat162*>(row + 46) = __floats2bfloat162_rn(f[4], f[5]);
  const __nv_bfloat162 z = __floats2bfloat162_rn(0.f, 0.f);
  for (int j = 48; j < kMlpInPad; j += 2) *reinterpret_cast<__nv_bfloat162*>(row + j) = z;
}

int launch_desc(int N, const float* rec, int64_t n, float* desc, cudaStream_t s);
int launch_datagen(int N, const float* rec, const float* box, const float* desc, int64_t n_elem, int64_t n,
                   uint64_t seed, void* X, float* T, uint8_t* V, cudaStream_t s);

}  // namespace ho
