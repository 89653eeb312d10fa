// The small network of the learned mode: 48 -> 128 -> 128 -> 128 -> 8,
// GELU (tanh form) after each hidden layer; BF16 operands, FP32 accumulation
// on the tensor cores (mma.sync m16n8k16), FP32 master weights with Adam.
//
//  * gemm_bf16<TA,TB>: C (+)= op(A) op(B) over row-major operands, 64x64
//    tiles, 4 warps x (16 rows x 64 cols), used by training (forward,
//    input-gradient and weight-gradient products).
//  * mlp_infer_kernel: the whole forward pass for inference, persistent over
//    128-row tiles, weights resident in shared memory, each warp owning 16
//    rows through all four layers (no block-level synchronisation between
//    layers).
//
// Weight layout: W_l[in][out] row-major (FP32 master and a BF16 copy), plus a
// BF16 transposed copy Wt_l[out][in] for the inference kernel's B operands.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include "ho_host.h"
#include "ho_mlp.h"
#include "ho_mlp_infer.cuh"

namespace ho {

// ---------------------------------------------------------------------------
// Generic GEMM for training. op(A)(m,k) = TA ? A[k*lda+m] : A[m*lda+k];
// op(B)(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n]. C row-major FP32.
// ---------------------------------------------------------------------------
constexpr int kGT = 64, kGK = 32, kGPad = 8;

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) gemm_bf16(int M, int N, int K, const bf16* __restrict__ A, int lda,
                                                 const bf16* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                                 int accumulate) {
  __shared__ __align__(16) bf16 As[kGT][kGK + kGPad];
  __shared__ __align__(16) bf16 Bs[kGT][kGK + kGPad];
  const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i][0] = acc[i][1] = acc[i][2] = acc[i][3] = 0.f;
  const bf16 zero = __float2bfloat16(0.f);
  // split-K: block z takes K range [kb, ke); partial sums are added atomically
  const int kchunk = (K + gridDim.z - 1) / gridDim.z;
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  for (int k0 = kb; k0 < ke; k0 += kGK) {
    for (int q = threadIdx.x; q < kGT * kGK; q += 128) {
      const int r = q / kGK, kk = q % kGK;
      const int m = m0 + r, k = k0 + kk, n = n0 + r;
      As[r][kk] = (m < M && k < ke) ? (TA ? A[static_cast<int64_t>(k) * lda + m] : A[static_cast<int64_t>(m) * lda + k])
                                    : zero;
      Bs[r][kk] = (n < N && k < ke) ? (TB ? B[static_cast<int64_t>(n) * ldb + k] : B[static_cast<int64_t>(k) * ldb + n])
                                    : zero;
    }
    __syncthreads();
    warp_mma<8>(&As[16 * warp][0], kGK + kGPad, &Bs[0][0], kGK + kGPad, kGK, acc);
    __syncthreads();
  }
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int m = m0 + 16 * warp + g + 8 * h;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int n = n0 + nt * 8 + 2 * t + c;
        if (m < M && n < N) {
          float* p = C + static_cast<int64_t>(m) * ldc + n;
          if (gridDim.z > 1) atomicAdd(p, acc[nt][2 * h + c]);
          else *p = accumulate ? *p + acc[nt][2 * h + c] : acc[nt][2 * h + c];
        }
      }
    }
  }
}

template <bool TA, bool TB>
static void gemm(cudaStream_t s, int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb, float* C, int ldc,
                 bool accumulate) {
  const int tiles = ((N + kGT - 1) / kGT) * ((M + kGT - 1) / kGT);
  // long reductions over few output tiles (weight gradients) are split over K
  int split = 1;
  if (K >= 1024 && tiles < 64) split = std::min(K / 256, 64 / tiles);
  if (split > 1 && !accumulate) cudaMemsetAsync(C, 0, sizeof(float) * static_cast<size_t>(M) * ldc, s);
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, split);
  gemm_bf16<TA, TB><<<grid, 128, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, accumulate ? 1 : 0);
}

// Z += bias; H = bf16(GELU(Z)) (or bf16(Z) for the output layer)
__global__ void bias_act_kernel(float* __restrict__ Z, const float* __restrict__ b, int M, int N,
                                bf16* __restrict__ H, int act) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<int64_t>(M) * N) return;
  const float z = Z[i] + b[i % N];
  Z[i] = z;
  if (H) H[i] = __float2bfloat16(act ? gelu(z) : z);
}

// dZ = bf16(dH * GELU'(Z))
__global__ void gelu_back_kernel(const float* __restrict__ dH, const float* __restrict__ Z, int64_t n,
                                 bf16* __restrict__ dZ, float* __restrict__ dZf) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = dH[i] * gelu_grad(Z[i]);
  dZ[i] = __float2bfloat16(v);
  dZf[i] = v;
}

// Masked MSE over the first kMlpTargets outputs: loss = mean over valid rows
// of sum_j (y_j - t_j)^2; dY = 2 (y - t) / n_valid.
__global__ void loss_kernel(const float* __restrict__ Y, const float* __restrict__ T, const uint8_t* __restrict__ valid,
                            int M, float inv_n, bf16* __restrict__ dY, float* __restrict__ dYf, float* loss) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<int64_t>(M) * kMlpOut) return;
  const int64_t r = i / kMlpOut;
  const int j = static_cast<int>(i % kMlpOut);
  float g = 0.f;
  if (j < kMlpTargets && valid[r]) {
    const float d = Y[i] - T[i];
    g = 2.f * d * inv_n;
    atomicAdd(loss, d * d * inv_n);
  }
  dY[i] = __float2bfloat16(g);
  dYf[i] = g;
}

// out[n] += sum over rows of D[m][n]; block b sums rows [256 b, 256 b + 256)
__global__ void colsum_kernel(const float* __restrict__ D, int M, int N, float* __restrict__ out) {
  const int n = threadIdx.x;
  if (n >= N) return;
  const int m0 = blockIdx.x * 256, m1 = min(M, m0 + 256);
  float s = 0.f;
  for (int m = m0; m < m1; ++m) s += D[static_cast<int64_t>(m) * N + n];
  atomicAdd(out + n, s);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2,
                            bf16* __restrict__ pb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  p[i] = pi;
  if (pb) pb[i] = __float2bfloat16(pi);
}

__global__ void gather_rows_kernel(const bf16* __restrict__ X, const float* __restrict__ T,
                                   const uint8_t* __restrict__ V, const int32_t* __restrict__ idx, int B,
                                   bf16* __restrict__ Xb, float* __restrict__ Tb, uint8_t* __restrict__ Vb) {
  const int r = blockIdx.x;
  if (r >= B) return;
  const int64_t s = idx[r];
  for (int c = threadIdx.x; c < kMlpInPad; c += blockDim.x) Xb[static_cast<int64_t>(r) * kMlpInPad + c] = X[s * kMlpInPad + c];
  for (int c = threadIdx.x; c < kMlpOut; c += blockDim.x) Tb[static_cast<int64_t>(r) * kMlpOut + c] = T[s * kMlpOut + c];
  if (threadIdx.x == 0) Vb[r] = V[s];
}

__global__ void transpose_cast_kernel(const float* __restrict__ W, int in, int out, int in_pad, int out_pad,
                                      bf16* __restrict__ Wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= in_pad * out_pad) return;
  const int o = i / in_pad, k = i % in_pad;
  Wt[i] = __float2bfloat16((o < out && k < in) ? W[k * out + o] : 0.f);
}

// ---------------------------------------------------------------------------
// Fused inference: Y[M x 8] = MLP(X[M x 64]) (X: 48 features + zero pad).
// ---------------------------------------------------------------------------
// Y[M x 8] = MLP(X[M x 64]) (X: 48 features + zero pad); M from m_dev
// (items x rows_per_item) when given.
__global__ void __launch_bounds__(256) mlp_infer_kernel(MlpDev P, const bf16* __restrict__ X, int64_t M,
                                                        const unsigned* __restrict__ m_dev, int rows_per_item,
                                                        float* __restrict__ Y) {
  const int64_t rows = m_dev ? static_cast<int64_t>(*m_dev) * rows_per_item : M;
  mlp_infer_tiles(P, XRows{X}, rows, Y);
}

size_t mlp_infer_smem() { return sizeof(InferSmem); }

int mlp_infer(const MlpDev& P, const void* X, int64_t M, const unsigned* m_dev, int rows_per_item, float* Y,
              cudaStream_t s, int grid) {
  // the attribute is set once per device
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return int(e);
  if (dev < 0 || dev >= 64) return int(cudaErrorInvalidDevice);
  if (!attr[dev].load(std::memory_order_acquire)) {
    e = cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(sizeof(InferSmem)));
    if (e != cudaSuccess) return int(e);
    attr[dev].store(true, std::memory_order_release);
  }
  mlp_infer_kernel<<<grid, 256, sizeof(InferSmem), s>>>(P, static_cast<const bf16*>(X), M, m_dev, rows_per_item, Y);
  return int(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Trainer
// ---------------------------------------------------------------------------
static const int kDims[5] = {kMlpInPad, kMlpHidden, kMlpHidden, kMlpHidden, kMlpOut};

#define MLP_TRY(x)                           \
  do {                                       \
    cudaError_t e__ = (x);                   \
    if (e__ != cudaSuccess) return int(e__); \
  } while (0)

int Mlp::alloc() {
  if (ready) return 0;
  for (int l = 0; l < 4; ++l) {
    const int n = kDims[l] * kDims[l + 1];
    MLP_TRY(cudaMalloc(&W[l], n * sizeof(float)));
    MLP_TRY(cudaMalloc(&Wb[l], n * sizeof(bf16)));
    MLP_TRY(cudaMalloc(&gW[l], n * sizeof(float)));
    MLP_TRY(cudaMalloc(&mW[l], n * sizeof(float)));
    MLP_TRY(cudaMalloc(&vW[l], n * sizeof(float)));
    MLP_TRY(cudaMalloc(&b[l], kDims[l + 1] * sizeof(float)));
    MLP_TRY(cudaMalloc(&gb[l], kDims[l + 1] * sizeof(float)));
    MLP_TRY(cudaMalloc(&mb[l], kDims[l + 1] * sizeof(float)));
    MLP_TRY(cudaMalloc(&vb[l], kDims[l + 1] * sizeof(float)));
  }
  MLP_TRY(cudaMalloc(&wt[0], kMlpHidden * kMlpInPad * sizeof(bf16)));
  MLP_TRY(cudaMalloc(&wt[1], kMlpHidden * kMlpHidden * sizeof(bf16)));
  MLP_TRY(cudaMalloc(&wt[2], kMlpHidden * kMlpHidden * sizeof(bf16)));
  MLP_TRY(cudaMalloc(&wt[3], 16 * kMlpHidden * sizeof(bf16)));
  ready = true;
  return 0;
}

void Mlp::release() {
  for (int l = 0; l < 4; ++l) {
    cudaFree(W[l]); cudaFree(Wb[l]); cudaFree(gW[l]); cudaFree(mW[l]); cudaFree(vW[l]);
    cudaFree(b[l]); cudaFree(gb[l]); cudaFree(mb[l]); cudaFree(vb[l]); cudaFree(wt[l]);
    W[l] = gW[l] = mW[l] = vW[l] = b[l] = gb[l] = mb[l] = vb[l] = nullptr;
    Wb[l] = nullptr;
    wt[l] = nullptr;
  }
  cudaFree(ws);
  ws = nullptr;
  ws_rows = 0;
  ready = false;
  trained = false;
}

// Host-side parameter upload: W_l[in][out] row-major fp32 (in padded to 64
// for layer 0, rows 48..63 must be zero), b_l.
int Mlp::set_params(const float* const* Wh, const float* const* bh, cudaStream_t s) {
  MLP_TRY(cudaError_t(alloc()));
  for (int l = 0; l < 4; ++l) {
    const int n = kDims[l] * kDims[l + 1];
    MLP_TRY(cudaMemcpyAsync(W[l], Wh[l], n * sizeof(float), cudaMemcpyHostToDevice, s));
    MLP_TRY(cudaMemcpyAsync(b[l], bh[l], kDims[l + 1] * sizeof(float), cudaMemcpyHostToDevice, s));
    MLP_TRY(cudaMemsetAsync(mW[l], 0, n * sizeof(float), s));
    MLP_TRY(cudaMemsetAsync(vW[l], 0, n * sizeof(float), s));
    MLP_TRY(cudaMemsetAsync(mb[l], 0, kDims[l + 1] * sizeof(float), s));
    MLP_TRY(cudaMemsetAsync(vb[l], 0, kDims[l + 1] * sizeof(float), s));
  }
  step = 0;
  return refresh_copies(s);
}

int Mlp::get_params(float* const* Wh, float* const* bh, cudaStream_t s) {
  for (int l = 0; l < 4; ++l) {
    const int n = kDims[l] * kDims[l + 1];
    MLP_TRY(cudaMemcpyAsync(Wh[l], W[l], n * sizeof(float), cudaMemcpyDeviceToHost, s));
    MLP_TRY(cudaMemcpyAsync(bh[l], b[l], kDims[l + 1] * sizeof(float), cudaMemcpyDeviceToHost, s));
  }
  return int(cudaStreamSynchronize(s));
}

__global__ void cast_kernel(const float* __restrict__ a, int n, bf16* __restrict__ o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = __float2bfloat16(a[i]);
}

int Mlp::refresh_copies(cudaStream_t s) {
  for (int l = 0; l < 4; ++l) {
    const int n = kDims[l] * kDims[l + 1];
    cast_kernel<<<(n + 255) / 256, 256, 0, s>>>(W[l], n, static_cast<bf16*>(Wb[l]));
  }
  transpose_cast_kernel<<<(kMlpHidden * kMlpInPad + 255) / 256, 256, 0, s>>>(W[0], kMlpInPad, kMlpHidden, kMlpInPad,
                                                                            kMlpHidden, static_cast<bf16*>(wt[0]));
  transpose_cast_kernel<<<(kMlpHidden * kMlpHidden + 255) / 256, 256, 0, s>>>(W[1], kMlpHidden, kMlpHidden,
                                                                             kMlpHidden, kMlpHidden, static_cast<bf16*>(wt[1]));
  transpose_cast_kernel<<<(kMlpHidden * kMlpHidden + 255) / 256, 256, 0, s>>>(W[2], kMlpHidden, kMlpHidden,
                                                                             kMlpHidden, kMlpHidden, static_cast<bf16*>(wt[2]));
  transpose_cast_kernel<<<(16 * kMlpHidden + 255) / 256, 256, 0, s>>>(W[3], kMlpHidden, kMlpOut, kMlpHidden, 16,
                                                                      static_cast<bf16*>(wt[3]));
  return int(cudaGetLastError());
}

MlpDev Mlp::dev() const {
  MlpDev d;
  d.w1t = wt[0];
  d.w2t = wt[1];
  d.w3t = wt[2];
  d.w4t = wt[3];
  d.b1 = b[0];
  d.b2 = b[1];
  d.b3 = b[2];
  d.b4 = b[3];
  return d;
}

int Mlp::ensure_ws(int rows) {
  if (rows <= ws_rows) return 0;
  cudaFree(ws);
  ws = nullptr;
  // Z1..Z3, dH, dZf: fp32 rows x 128 each (5); Y, dYf: rows x 8 (2);
  // H0(X), H1..H3, dZ bf16: rows x 128 (5, X padded to 64 inside); dY bf16 rows x 8; T rows x 8; valid rows
  const size_t f32 = static_cast<size_t>(rows) * (5 * kMlpHidden + 3 * kMlpOut) * sizeof(float);
  const size_t b16 = static_cast<size_t>(rows) * (5 * kMlpHidden + kMlpOut) * sizeof(bf16);
  MLP_TRY(cudaMalloc(&ws, f32 + b16 + rows + 64));
  ws_rows = rows;
  return 0;
}

// Forward + backward on a batch already in the workspace layout; gradients
// overwrite gW/gb; returns the batch loss through loss_dev.
int Mlp::forward_backward(int B, const void* Xb, const float* Tb, const uint8_t* Vb, int n_valid, float* loss_dev,
                          cudaStream_t s) {
  MLP_TRY(cudaError_t(ensure_ws(B)));
  float* f = static_cast<float*>(ws);
  float* Z[3] = {f, f + static_cast<size_t>(B) * kMlpHidden, f + 2 * static_cast<size_t>(B) * kMlpHidden};
  float* dH = f + 3 * static_cast<size_t>(B) * kMlpHidden;
  float* dZf = f + 4 * static_cast<size_t>(B) * kMlpHidden;
  float* Y = f + 5 * static_cast<size_t>(B) * kMlpHidden;
  float* dYf = Y + static_cast<size_t>(B) * kMlpOut;
  bf16* hb = reinterpret_cast<bf16*>(dYf + 2 * static_cast<size_t>(B) * kMlpOut);
  bf16* H[3] = {hb, hb + static_cast<size_t>(B) * kMlpHidden, hb + 2 * static_cast<size_t>(B) * kMlpHidden};
  bf16* dZ = hb + 3 * static_cast<size_t>(B) * kMlpHidden;
  bf16* dY = hb + 4 * static_cast<size_t>(B) * kMlpHidden;
  const bf16* X = static_cast<const bf16*>(Xb);
  const int th = 256;
  auto blocks = [&](int64_t n) { return static_cast<unsigned>((n + th - 1) / th); };
  // forward
  const bf16* in = X;
  int in_dim = kMlpInPad;
  for (int l = 0; l < 3; ++l) {
    gemm<false, false>(s, B, kMlpHidden, in_dim, in, in_dim, static_cast<const bf16*>(Wb[l]), kMlpHidden, Z[l], kMlpHidden, false);
    bias_act_kernel<<<blocks(static_cast<int64_t>(B) * kMlpHidden), th, 0, s>>>(Z[l], b[l], B, kMlpHidden, H[l], 1);
    in = H[l];
    in_dim = kMlpHidden;
  }
  gemm<false, false>(s, B, kMlpOut, kMlpHidden, H[2], kMlpHidden, static_cast<const bf16*>(Wb[3]), kMlpOut, Y, kMlpOut, false);
  bias_act_kernel<<<blocks(static_cast<int64_t>(B) * kMlpOut), th, 0, s>>>(Y, b[3], B, kMlpOut, nullptr, 0);
  MLP_TRY(cudaMemsetAsync(loss_dev, 0, sizeof(float), s));
  loss_kernel<<<blocks(static_cast<int64_t>(B) * kMlpOut), th, 0, s>>>(Y, Tb, Vb, B, 1.0f / std::max(1, n_valid), dY,
                                                                       dYf, loss_dev);
  // backward: layer 3 (output)
  for (int l = 0; l < 4; ++l) {
    MLP_TRY(cudaMemsetAsync(gb[l], 0, kDims[l + 1] * sizeof(float), s));
  }
  gemm<true, false>(s, kMlpHidden, kMlpOut, B, H[2], kMlpHidden, dY, kMlpOut, gW[3], kMlpOut, false);
  colsum_kernel<<<(B + 255) / 256, kMlpOut, 0, s>>>(dYf, B, kMlpOut, gb[3]);
  gemm<false, true>(s, B, kMlpHidden, kMlpOut, dY, kMlpOut, static_cast<const bf16*>(Wb[3]), kMlpOut, dH, kMlpHidden, false);
  for (int l = 2; l >= 0; --l) {
    gelu_back_kernel<<<blocks(static_cast<int64_t>(B) * kMlpHidden), th, 0, s>>>(dH, Z[l],
                                                                                static_cast<int64_t>(B) * kMlpHidden,
                                                                                dZ, dZf);
    const bf16* a_in = l > 0 ? H[l - 1] : X;
    const int a_dim = l > 0 ? kMlpHidden : kMlpInPad;
    gemm<true, false>(s, a_dim, kMlpHidden, B, a_in, a_dim, dZ, kMlpHidden, gW[l], kMlpHidden, false);
    colsum_kernel<<<(B + 255) / 256, kMlpHidden, 0, s>>>(dZf, B, kMlpHidden, gb[l]);
    if (l > 0) gemm<false, true>(s, B, kMlpHidden, kMlpHidden, dZ, kMlpHidden, static_cast<const bf16*>(Wb[l]), kMlpHidden, dH, kMlpHidden, false);
  }
  return int(cudaGetLastError());
}

int Mlp::adam_step(float lr, cudaStream_t s) {
  ++step;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - std::pow(b1, static_cast<float>(step)), c2 = 1.f - std::pow(b2, static_cast<float>(step));
  for (int l = 0; l < 4; ++l) {
    const int n = kDims[l] * kDims[l + 1];
    adam_kernel<<<(n + 255) / 256, 256, 0, s>>>(W[l], gW[l], mW[l], vW[l], n, lr, b1, b2, eps, c1, c2,
                                                static_cast<bf16*>(Wb[l]));
    adam_kernel<<<(kDims[l + 1] + 255) / 256, 256, 0, s>>>(b[l], gb[l], mb[l], vb[l], kDims[l + 1], lr, b1, b2, eps,
                                                            c1, c2, nullptr);
  }
  return int(cudaGetLastError());
}

// Layer 0 rows 48..63 are the zero padding of the input: keep them zero.
__global__ void zero_pad_rows_kernel(float* W0, float* m0, float* v0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = (kMlpInPad - kMlpIn) * kMlpHidden;
  if (i >= n) return;
  const int off = kMlpIn * kMlpHidden + i;
  W0[off] = 0.f;
  m0[off] = 0.f;
  v0[off] = 0.f;
}

int Mlp::train(const void* X, const float* T, const uint8_t* V, int64_t n, int steps, int batch, float lr, uint64_t seed,
               std::vector<float>& losses, cudaStream_t s) {
  MLP_TRY(cudaError_t(ensure_ws(batch)));
  bf16* Xb;
  float* Tb;
  uint8_t* Vb;
  int32_t* idx;
  float* loss_dev;
  MLP_TRY(cudaMalloc(&Xb, static_cast<size_t>(batch) * kMlpInPad * sizeof(bf16)));
  MLP_TRY(cudaMalloc(&Tb, static_cast<size_t>(batch) * kMlpOut * sizeof(float)));
  MLP_TRY(cudaMalloc(&Vb, batch));
  MLP_TRY(cudaMalloc(&idx, batch * sizeof(int32_t)));
  MLP_TRY(cudaMalloc(&loss_dev, sizeof(float)));
  std::vector<int32_t> hidx(batch);
  Pcg64 rng(seed, 7);
  losses.clear();
  float* hloss = nullptr;
  MLP_TRY(cudaMallocHost(&hloss, sizeof(float) * std::max(1, steps)));
  for (int it = 0; it < steps; ++it) {
    for (int i = 0; i < batch; ++i) hidx[i] = static_cast<int32_t>(rng.next() % static_cast<uint64_t>(n));
    MLP_TRY(cudaMemcpyAsync(idx, hidx.data(), batch * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    gather_rows_kernel<<<batch, 64, 0, s>>>(static_cast<const bf16*>(X), T, V, idx, batch, Xb, Tb, Vb);
    // cosine decay to 5% of lr
    const float lr_t = lr * (0.05f + 0.95f * 0.5f * (1.f + std::cos(3.14159265f * it / std::max(1, steps))));
    int rc = forward_backward(batch, Xb, Tb, Vb, batch, loss_dev, s);
    if (rc) return rc;
    rc = adam_step(lr_t, s);
    if (rc) return rc;
    zero_pad_rows_kernel<<<((kMlpInPad - kMlpIn) * kMlpHidden + 255) / 256, 256, 0, s>>>(W[0], mW[0], vW[0]);
    MLP_TRY(cudaMemcpyAsync(hloss + it, loss_dev, sizeof(float), cudaMemcpyDeviceToHost, s));
    // host copy of the loss waits for the stream only at the end
  }
  MLP_TRY(cudaStreamSynchronize(s));
  losses.assign(hloss, hloss + steps);
  cudaFreeHost(hloss);
  cudaFree(Xb);
  cudaFree(Tb);
  cudaFree(Vb);
  cudaFree(idx);
  cudaFree(loss_dev);
  const int rc = refresh_copies(s);
  if (rc) return rc;
  trained = true;
  return 0;
}

}  // namespace ho
