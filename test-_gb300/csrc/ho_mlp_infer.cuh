// The learned mode's network inference (48 -> 128 -> 128 -> 128 -> 8, GELU
// in tanh form after each hidden layer, BF16 operands, FP32 accumulation on
// mma.sync m16n8k16) as a device routine over a caller-defined source of
// input rows, so that the input rows can be formed inside the kernel that
// runs the network (ho_trace.cu) or read from memory (ho_mlp.cu), and the
// tensor-core helpers shared with the trainer's GEMMs.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "ho_mlp.h"

namespace ho {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// One warp: acc[nt] += A[16 x K] * B[K x 8*NT]; A row-major in shared memory
// (row stride lda elements), B given as Bt[n][k] (stride ldb). K % 16 == 0.
// Fragment layout of m16n8k16 (g = lane/4, t = lane%4): A regs = rows g and
// g+8, k pairs 2t and 2t+8; B regs = column g, k pairs 2t and 2t+8; C = rows
// g and g+8, columns 2t, 2t+1.
template <int NT>
__device__ __forceinline__ void warp_mma(const bf16* A, int lda, const bf16* Bt, int ldb, int K, float (&acc)[NT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  for (int k0 = 0; k0 < K; k0 += 16) {
    const uint32_t a0 = ld32(A + g * lda + k0 + 2 * t);
    const uint32_t a1 = ld32(A + (g + 8) * lda + k0 + 2 * t);
    const uint32_t a2 = ld32(A + g * lda + k0 + 2 * t + 8);
    const uint32_t a3 = ld32(A + (g + 8) * lda + k0 + 2 * t + 8);
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const bf16* bp = Bt + (nt * 8 + g) * ldb + k0 + 2 * t;
      mma_bf16(acc[nt], a0, a1, a2, a3, ld32(bp), ld32(bp + 8));
    }
  }
}

// GELU in its tanh form (Hendrycks and Gimpel): 0.5 x (1 + tanh(a (x + b x^3)))
// with a = sqrt(2 / pi), b = 0.044715. Training uses tanhf; inference the
// hardware approximation (tanh.approx.f32, one instruction, relative error
// about 2^-11, below the BF16 rounding of the activations it feeds).
constexpr float kGeluA = 0.7978845608028654f, kGeluB = 0.044715f;
__device__ __forceinline__ float gelu_arg(float x) { return kGeluA * fmaf(kGeluB * x, x * x, x); }
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + tanhf(gelu_arg(x))); }
__device__ __forceinline__ float gelu_fast(float x) {
  float th;
  asm("tanh.approx.f32 %0, %1;" : "=f"(th) : "f"(gelu_arg(x)));
  const float h = 0.5f * x;
  return fmaf(h, th, h);
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float th = tanhf(gelu_arg(x));
  return 0.5f * (1.0f + th) + 0.5f * x * (1.0f - th * th) * kGeluA * fmaf(3.0f * kGeluB, x * x, 1.0f);
}

struct InferSmem {
  bf16 w1t[kMlpHidden][kMlpInPad + 8];
  bf16 w2t[kMlpHidden][kMlpHidden + 8];
  bf16 w3t[kMlpHidden][kMlpHidden + 8];
  bf16 w4t[16][kMlpHidden + 8];
  float b1[kMlpHidden], b2[kMlpHidden], b3[kMlpHidden], b4[16];
  bf16 x[128][kMlpInPad + 8];
  bf16 h0[128][kMlpHidden + 8];
  bf16 h1[128][kMlpHidden + 8];
};

template <int NT>
__device__ __forceinline__ void act_store(float (&acc)[NT][4], const float* bias, bf16* H, int ldh, int row0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = row0 + g + 8 * h, c = nt * 8 + 2 * t;
      const float v0 = gelu_fast(acc[nt][2 * h] + bias[c]);
      const float v1 = gelu_fast(acc[nt][2 * h + 1] + bias[c + 1]);
      *reinterpret_cast<__nv_bfloat162*>(H + r * ldh + c) = __floats2bfloat162_rn(v0, v1);
    }
}

// The forward pass over `rows` rows of network input, persistent over
// 128-row tiles: weights resident in shared memory, each warp owning 16 rows
// through all four layers (no block-level synchronisation between layers).
// R.fill(row, half, dst) writes half `half` (32 BF16) of the row's input.
template <class Rows>
__device__ __forceinline__ void mlp_infer_tiles(const MlpDev& P, const Rows& R, int64_t rows, float* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
  for (int i = threadIdx.x; i < kMlpHidden * kMlpInPad; i += blockDim.x)
    S.w1t[i / kMlpInPad][i % kMlpInPad] = static_cast<const bf16*>(P.w1t)[i];
  for (int i = threadIdx.x; i < kMlpHidden * kMlpHidden; i += blockDim.x) {
    S.w2t[i / kMlpHidden][i % kMlpHidden] = static_cast<const bf16*>(P.w2t)[i];
    S.w3t[i / kMlpHidden][i % kMlpHidden] = static_cast<const bf16*>(P.w3t)[i];
  }
  for (int i = threadIdx.x; i < 16 * kMlpHidden; i += blockDim.x) S.w4t[i / kMlpHidden][i % kMlpHidden] = static_cast<const bf16*>(P.w4t)[i];
  for (int i = threadIdx.x; i < kMlpHidden; i += blockDim.x) {
    S.b1[i] = P.b1[i];
    S.b2[i] = P.b2[i];
    S.b3[i] = P.b3[i];
  }
  for (int i = threadIdx.x; i < 16; i += blockDim.x) S.b4[i] = i < kMlpOut ? P.b4[i] : 0.f;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int r0 = 16 * warp;
  for (int64_t tile = blockIdx.x; tile * 128 < rows; tile += gridDim.x) {
    const int64_t base = tile * 128;
    // this warp's 16 rows of network input, two lanes per row
    {
      const int r = lane >> 1, half = lane & 1;
      const int64_t gr = base + r0 + r;
      bf16* dst = &S.x[r0 + r][half * (kMlpInPad / 2)];
      if (gr < rows) {
        R.fill(gr, half, dst);
      } else {
        const uint4 z = make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int q = 0; q < kMlpInPad / 16; ++q) reinterpret_cast<uint4*>(dst)[q] = z;
      }
    }
    __syncwarp();
    {
      float acc[16][4] = {};
      warp_mma<16>(&S.x[r0][0], kMlpInPad + 8, &S.w1t[0][0], kMlpInPad + 8, kMlpInPad, acc);
      act_store<16>(acc, S.b1, &S.h0[0][0], kMlpHidden + 8, r0);
    }
    __syncwarp();
    {
      float acc[16][4] = {};
      warp_mma<16>(&S.h0[r0][0], kMlpHidden + 8, &S.w2t[0][0], kMlpHidden + 8, kMlpHidden, acc);
      act_store<16>(acc, S.b2, &S.h1[0][0], kMlpHidden + 8, r0);
    }
    __syncwarp();
    {
      float acc[16][4] = {};
      warp_mma<16>(&S.h1[r0][0], kMlpHidden + 8, &S.w3t[0][0], kMlpHidden + 8, kMlpHidden, acc);
      act_store<16>(acc, S.b3, &S.h0[0][0], kMlpHidden + 8, r0);
    }
    __syncwarp();
    {
      float acc[2][4] = {};
      warp_mma<2>(&S.h0[r0][0], kMlpHidden + 8, &S.w4t[0][0], kMlpHidden + 8, kMlpHidden, acc);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t gr = base + r0 + g + 8 * h;
        const int c = 2 * t;  // n-tile 0 holds outputs 0..7
        if (gr < rows) {
          Y[gr * kMlpOut + c] = acc[0][2 * h] + S.b4[c];
          Y[gr * kMlpOut + c + 1] = acc[0][2 * h + 1] + S.b4[c + 1];
        }
      }
    }
    __syncwarp();
  }
}


// Input rows read from a row-major BF16 matrix X[rows][64].
struct XRows {
  const bf16* X;
  __device__ __forceinline__ void fill(int64_t row, int half, bf16* dst) const {
    const uint4* src = reinterpret_cast<const uint4*>(X + row * kMlpInPad + half * (kMlpInPad / 2));
#pragma unroll
    for (int q = 0; q < kMlpInPad / 16; ++q) reinterpret_cast<uint4*>(dst)[q] = src[q];
  }
};

}  // namespace ho
