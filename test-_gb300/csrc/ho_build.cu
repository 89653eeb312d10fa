// Scene set-up on the device: per-element boxes and the LBVH.
//
//  * padded sampled box: the box of max(4, n+2)^3 reference-grid points
//    padded by 15% of its size (at least 1e-3) — the box the reference uses
//    to admit a candidate and to bound its isosurface segment
//    (FEM-AABB/high_order.h:51-113); trilinear elements use their corners
//    padded by 1e-4 (high_order.h:59-76).
//  * hull box: min/max of the Bernstein control points of the element's
//    geometry over [-1,1]^3 — a rigorous bound of the curved element.
//  * face hull boxes: the same for each of the 6 faces over
//    [-1.001,1.001]^2 (the reference's face acceptance range), inflated past
//    the face Newton's 1e-4 tolerance; used to skip faces exactly.
//  * LBVH (Karras 2012): 30-bit Morton codes of box centres, a stable LSD
//    radix sort (8-bit digits), one kernel for the whole hierarchy, and a
//    bottom-up refit with per-node arrival counters. Replaces the reference's
//    host-side binned SAH build (FEM-AABB/BVH.cu:35-247).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ho_device.cuh"
#include "ho_host.h"

namespace ho {

#define HO_TRY(x)                          \
  do {                                     \
    cudaError_t e__ = (x);                 \
    if (e__ != cudaSuccess) return int(e__); \
  } while (0)

// Change-of-basis matrices (Modified-A -> Bernstein), row i = mode i.
struct BernMats {
  float cube[kMaxModes * kMaxModes];  // on [-1, 1]
  float face[kMaxModes * kMaxModes];  // on [-1.001, 1.001]
};

constexpr int kSetupWarps = 4;

// One warp per element.
template <int N>
__global__ void __launch_bounds__(32 * kSetupWarps) setup_kernel(const float* __restrict__ rec,
                                                                 const uint32_t* __restrict__ flags,
                                                                 const int32_t* __restrict__ own, int64_t n_elem,
                                                                 BernMats bm, float* __restrict__ box,
                                                                 float* __restrict__ hull, float* __restrict__ fbox) {
  constexpr int S = N * N * N;
  constexpr int RS = row_stride(N), BF = block_floats(N);
  __shared__ float sh[kSetupWarps][2 * S];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t e = static_cast<int64_t>(blockIdx.x) * kSetupWarps + wib;
  if (e >= n_elem) return;
  const float* r = rec + e * record_floats(N);
  Elem<N> el;
  el.c = CoefRef<false>{r};
  el.has_field = false;
  Work w;
  const bool tri = (flags[e] & 2u) != 0;
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  if (tri) {
    // corners sit at the N=2 modal slots (i,j,k) in {0,1}^3
    if (lane < 8) {
      const int i = lane & 1, j = (lane >> 1) & 1, k = lane >> 2;
      for (int c = 0; c < 3; ++c) {
        const float v = r[c * BF + (k * N + j) * RS + i];
        lo[c] = v;
        hi[c] = v;
      }
    }
  } else {
    const int ns = max(4, own[e] + 2);
    const int total = ns * ns * ns;
    for (int q = lane; q < total; q += 32) {
      const int kx = q % ns, ky = (q / ns) % ns, kz = q / (ns * ns);
      const float rx = -1.0f + 2.0f * static_cast<float>(kx) / static_cast<float>(ns - 1);
      const float sy = -1.0f + 2.0f * static_cast<float>(ky) / static_cast<float>(ns - 1);
      const float tz = -1.0f + 2.0f * static_cast<float>(kz) / static_cast<float>(ns - 1);
      const float3 p = geom_map<N>(el, make_float3(rx, sy, tz), w);
      lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
      hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], off));
      hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], off));
    }
  if (lane == 0) {
    float* b = box + 6 * e;
    if (tri) {
      for (int c = 0; c < 3; ++c) {
        b[c] = lo[c] - 1e-4f;
        b[3 + c] = hi[c] + 1e-4f;
      }
    } else {
      for (int c = 0; c < 3; ++c) {
        const float pad = fmaxf((hi[c] - lo[c]) * 0.15f, 1e-3f);
        b[c] = lo[c] - pad;
        b[3 + c] = hi[c] + pad;
      }
    }
  }

  // Bernstein hull of the element and of its faces, one component at a time.
  float* t0 = sh[wib];
  float* t1 = sh[wib] + S;
  float elo[3], ehi[3], flo[6][3], fhi[6][3];
  for (int c = 0; c < 3; ++c) {
    const float* src = r + c * BF;
    // faces: slices at the fixed axis' vertex mode, then 2-D transform
    for (int f = 0; f < 6; ++f) {
      int fixed, ua, va;
      float val;
      face_param(f, fixed, val, ua, va);
      const int m = val < 0.f ? 0 : 1;
      float mn = FLT_MAX, mxv = -FLT_MAX;
      for (int q = lane; q < N * N; q += 32) {
        const int bu = q % N, bv = q / N;  // output Bernstein indices
        float acc = 0.f;
        for (int iv = 0; iv < N; ++iv)
          for (int iu = 0; iu < N; ++iu) {
            int idx[3];
            idx[fixed] = m;
            idx[ua] = iu;
            idx[va] = iv;
            const float cv = src[(idx[2] * N + idx[1]) * RS + idx[0]];
            acc = fmaf(cv, bm.face[iu * kMaxModes + bu] * bm.face[iv * kMaxModes + bv], acc);
          }
        mn = fminf(mn, acc);
        mxv = fmaxf(mxv, acc);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
        mxv = fmaxf(mxv, __shfl_xor_sync(0xffffffffu, mxv, off));
      }
      flo[f][c] = mn;
      fhi[f][c] = mxv;
    }
    // element: three 1-D passes through shared memory
    for (int q = lane; q < S; q += 32) {
      const int b = q % N, j = (q / N) % N, k = q / (N * N);
      float acc = 0.f;
      for (int i = 0; i < N; ++i) acc = fmaf(src[(k * N + j) * RS + i], bm.cube[i * kMaxModes + b], acc);
      t0[q] = acc;
    }
    __syncwarp();
    for (int q = lane; q < S; q += 32) {
      const int a = q % N, b = (q / N) % N, k = q / (N * N);
      float acc = 0.f;
      for (int j = 0; j < N; ++j) acc = fmaf(t0[(k * N + j) * N + a], bm.cube[j * kMaxModes + b], acc);
      t1[q] = acc;
    }
    __syncwarp();
    float mn = FLT_MAX, mxv = -FLT_MAX;
    for (int q = lane; q < S; q += 32) {
      const int a = q % N, b = (q / N) % N, cc = q / (N * N);
      float acc = 0.f;
      for (int k = 0; k < N; ++k) acc = fmaf(t1[(k * N + b) * N + a], bm.cube[k * kMaxModes + cc], acc);
      mn = fminf(mn, acc);
      mxv = fmaxf(mxv, acc);
    }
    __syncwarp();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mxv = fmaxf(mxv, __shfl_xor_sync(0xffffffffu, mxv, off));
    }
    elo[c] = mn;
    ehi[c] = mxv;
  }
  if (lane == 0) {
    for (int c = 0; c < 3; ++c) {
      const float m = 1e-6f * (1.0f + fabsf(elo[c]) + fabsf(ehi[c]));
      hull[6 * e + c] = elo[c] - m;
      hull[6 * e + 3 + c] = ehi[c] + m;
    }
    for (int f = 0; f < 6; ++f)
      for (int c = 0; c < 3; ++c) {
        // face acceptance tolerance 1e-4 (max-norm residual) + rounding
        const float m = 2.5e-4f + 1e-5f * (fabsf(flo[f][c]) + fabsf(fhi[f][c]));
        fbox[kFaceBoxFloats * e + 6 * f + c] = flo[f][c] - m;
        fbox[kFaceBoxFloats * e + 6 * f + 3 + c] = fhi[f][c] + m;
      }
  }
}

template <int N>
static cudaError_t launch_setup_n(ho_context* c, const BernMats& bm) {
  const int64_t blocks = (c->n_elem + kSetupWarps - 1) / kSetupWarps;
  setup_kernel<N><<<static_cast<unsigned>(blocks), 32 * kSetupWarps, 0, c->stream>>>(
      c->d_rec, c->d_flags, c->d_own, c->n_elem, bm, c->d_box, c->d_hull, c->d_fbox);
  return cudaGetLastError();
}

int launch_setup(ho_context* c) {
  BernMats bm;
  std::memset(&bm, 0, sizeof(bm));
  std::vector<double> M;
  modal_to_bernstein(c->N, -1.0, 1.0, M);
  for (int i = 0; i < c->N; ++i)
    for (int k = 0; k < c->N; ++k) bm.cube[i * kMaxModes + k] = static_cast<float>(M[i * c->N + k]);
  modal_to_bernstein(c->N, -1.001, 1.001, M);
  for (int i = 0; i < c->N; ++i)
    for (int k = 0; k < c->N; ++k) bm.face[i * kMaxModes + k] = static_cast<float>(M[i * c->N + k]);
  cudaError_t e;
  switch (c->N) {
    case 2: e = launch_setup_n<2>(c, bm); break;
    case 3: e = launch_setup_n<3>(c, bm); break;
    case 4: e = launch_setup_n<4>(c, bm); break;
    case 5: e = launch_setup_n<5>(c, bm); break;
    case 6: e = launch_setup_n<6>(c, bm); break;
    case 7: e = launch_setup_n<7>(c, bm); break;
    case 8: e = launch_setup_n<8>(c, bm); break;
    case 9: e = launch_setup_n<9>(c, bm); break;
    default: return int(cudaErrorInvalidValue);
  }
  return int(e);
}

// ---------------------------------------------------------------------------
// LBVH
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void morton_kernel(const float* __restrict__ box, int64_t n, float3 lo, float3 inv_ext,
                              uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* b = box + 6 * i;
  const float cx = 0.5f * (b[0] + b[3]), cy = 0.5f * (b[1] + b[4]), cz = 0.5f * (b[2] + b[5]);
  const float fx = fminf(fmaxf((cx - lo.x) * inv_ext.x, 0.f), 1.f);
  const float fy = fminf(fmaxf((cy - lo.y) * inv_ext.y, 0.f), 1.f);
  const float fz = fminf(fmaxf((cz - lo.z) * inv_ext.z, 0.f), 1.f);
  const uint32_t qx = min(static_cast<uint32_t>(fx * 1024.f), 1023u);
  const uint32_t qy = min(static_cast<uint32_t>(fy * 1024.f), 1023u);
  const uint32_t qz = min(static_cast<uint32_t>(fz * 1024.f), 1023u);
  keys[i] = (spread10(qx) << 2) | (spread10(qy) << 1) | spread10(qz);
  vals[i] = static_cast<int32_t>(i);
}

constexpr int kSortTile = 256;

__global__ void __launch_bounds__(kSortTile) radix_hist_kernel(const uint32_t* __restrict__ keys, int64_t n, int shift,
                                                               int n_tiles, uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kSortTile + threadIdx.x;
  if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[static_cast<int64_t>(threadIdx.x) * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of len values with one block of 1024 threads, in tiles of
// 4096 (4 consecutive values per thread, warp shuffles, then the 32 warp
// totals), carrying the running total from tile to tile.
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t* __restrict__ data, int64_t len) {
  __shared__ uint32_t wsum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t carry = 0;
  for (int64_t base = 0; base < len; base += 4096) {
    const int64_t i0 = base + static_cast<int64_t>(threadIdx.x) * 4;
    uint32_t v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = i0 + k < len ? data[i0 + k] : 0u;
    const uint32_t t = v[0] + v[1] + v[2] + v[3];
    uint32_t x = t;  // inclusive scan over the warp
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint32_t ws = wsum[lane];
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, ws, off);
        if (lane >= off) ws += y;
      }
      wsum[lane] = ws;
    }
    __syncthreads();
    uint32_t run = carry + (wid > 0 ? wsum[wid - 1] : 0u) + (x - t);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (i0 + k < len) data[i0 + k] = run;
      run += v[k];
    }
    carry += wsum[31];
    __syncthreads();  // every thread has read wsum before the next tile writes it
  }
}

// Stable scatter: rank among equal digits inside the tile via warp matching.
__global__ void __launch_bounds__(kSortTile) radix_scatter_kernel(const uint32_t* __restrict__ kin,
                                                                  const int32_t* __restrict__ vin, int64_t n,
                                                                  int shift, int n_tiles,
                                                                  const uint32_t* __restrict__ offs,
                                                                  uint32_t* __restrict__ kout,
                                                                  int32_t* __restrict__ vout) {
  constexpr int W = kSortTile / 32;
  __shared__ uint32_t wcnt[W][256];
  __shared__ uint32_t woff[W][256];
  for (int q = threadIdx.x; q < W * 256; q += kSortTile) (&wcnt[0][0])[q] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kSortTile + threadIdx.x;
  const bool valid = i < n;
  const uint32_t key = valid ? kin[i] : 0u;
  const uint32_t dig = valid ? ((key >> shift) & 255u) : (256u + lane);
  const uint32_t peers = __match_any_sync(0xffffffffu, dig);
  const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
  if (valid && rank == 0) wcnt[wid][dig] = __popc(peers);
  __syncthreads();
  {
    uint32_t run = 0;
    for (int w = 0; w < W; ++w) {
      const uint32_t v = wcnt[w][threadIdx.x];
      woff[w][threadIdx.x] = run;
      run += v;
    }
  }
  __syncthreads();
  if (valid) {
    const uint32_t pos = offs[static_cast<int64_t>(dig) * n_tiles + blockIdx.x] + woff[wid][dig] + rank;
    kout[pos] = key;
    vout[pos] = vin[i];
  }
}

__device__ __forceinline__ int delta(const uint32_t* __restrict__ k, int64_t n, int64_t i, int64_t j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = k[i], b = k[j];
  if (a == b) return 32 + __clz(static_cast<uint32_t>(i ^ j));
  return __clz(a ^ b);
}

__global__ void karras_kernel(const uint32_t* __restrict__ k, const int32_t* __restrict__ vals,
                              const uint32_t* __restrict__ eflags, int64_t n, BNode* __restrict__ nodes,
                              int32_t* __restrict__ parent_int, int32_t* __restrict__ parent_leaf) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(k, n, i, i - d);
  int64_t lmax = 2;
  while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int64_t l = 0;
  for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  const int64_t j = i + l * d;
  const int dnode = delta(k, n, i, j);
  int64_t s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int64_t g = i + s * d + min(d, 0);
  const int64_t lo = min(i, j), hi = max(i, j);
  BNode nd;
  for (int c = 0; c < 2; ++c) {
    for (int a = 0; a < 3; ++a) {
      nd.c[c].lo[a] = FLT_MAX;
      nd.c[c].hi[a] = -FLT_MAX;
    }
    nd.c[c].aux = 0;
  }
  if (lo == g) {
    const int32_t e = vals[g];
    nd.c[0].idx = ~e;
    nd.c[0].aux = eflags ? (eflags[e] & kAuxHasField) : 0u;
    parent_leaf[g] = static_cast<int32_t>(i);
  } else {
    nd.c[0].idx = static_cast<int32_t>(g);
    parent_int[g] = static_cast<int32_t>(i);
  }
  if (hi == g + 1) {
    const int32_t e = vals[g + 1];
    nd.c[1].idx = ~e;
    nd.c[1].aux = eflags ? (eflags[e] & kAuxHasField) : 0u;
    parent_leaf[g + 1] = static_cast<int32_t>(i);
  } else {
    nd.c[1].idx = static_cast<int32_t>(g + 1);
    parent_int[g + 1] = static_cast<int32_t>(i);
  }
  nodes[i] = nd;
}

__global__ void refit_kernel(const float* __restrict__ box, const int32_t* __restrict__ vals, int64_t n,
                             BNode* nodes, const int32_t* __restrict__ parent_int,
                             const int32_t* __restrict__ parent_leaf, uint32_t* __restrict__ arrive) {
  const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int32_t e = vals[p];
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = box[6 * e + a];
    hi[a] = box[6 * e + 3 + a];
  }
  int32_t node = parent_leaf[p];
  int32_t me = ~e;
  while (node >= 0) {
    ChildRec* cr = nodes[node].c;
    const int slot = (__ldcg(&cr[0].idx) == me) ? 0 : 1;
    for (int a = 0; a < 3; ++a) {
      cr[slot].lo[a] = lo[a];
      cr[slot].hi[a] = hi[a];
    }
    __threadfence();
    if (atomicAdd(&arrive[node], 1u) == 0) return;  // sibling not done yet
    __threadfence();
    for (int a = 0; a < 3; ++a) {
      lo[a] = fminf(__ldcg(&cr[0].lo[a]), __ldcg(&cr[1].lo[a]));
      hi[a] = fmaxf(__ldcg(&cr[0].hi[a]), __ldcg(&cr[1].hi[a]));
    }
    me = node;
    node = node == 0 ? -1 : parent_int[node];
  }
}

int build_lbvh(ho_context* c) {
  return build_tree(c->d_box, c->d_flags, c->n_elem, c->stream, &c->d_nodes, &c->n_nodes, &c->bvh_depth, c->bounds);
}

int build_tree(const float* d_box, const uint32_t* d_flags, int64_t n, cudaStream_t s, BNode** nodes_out,
               int64_t* n_nodes_out, int* depth_out, float bounds[6]) {
  // scene bounds over box centres (host; the boxes are small)
  std::vector<float> hb(static_cast<size_t>(n) * 6);
  HO_TRY(cudaMemcpyAsync(hb.data(), d_box, hb.size() * sizeof(float), cudaMemcpyDeviceToHost, s));
  HO_TRY(cudaStreamSynchronize(s));
  float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int a = 0; a < 3; ++a) {
    bounds[a] = FLT_MAX;
    bounds[3 + a] = -FLT_MAX;
  }
  for (int64_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      const float cc = 0.5f * (hb[6 * i + a] + hb[6 * i + 3 + a]);
      clo[a] = std::min(clo[a], cc);
      chi[a] = std::max(chi[a], cc);
      bounds[a] = std::min(bounds[a], hb[6 * i + a]);
      bounds[3 + a] = std::max(bounds[3 + a], hb[6 * i + 3 + a]);
    }
  const float3 lo = make_float3(clo[0], clo[1], clo[2]);
  const float3 inv = make_float3(chi[0] > clo[0] ? 1.f / (chi[0] - clo[0]) : 0.f,
                                 chi[1] > clo[1] ? 1.f / (chi[1] - clo[1]) : 0.f,
                                 chi[2] > clo[2] ? 1.f / (chi[2] - clo[2]) : 0.f);

  const int64_t n_nodes = std::max<int64_t>(1, n - 1);
  *n_nodes_out = n_nodes;
  HO_TRY(cudaMalloc(nodes_out, n_nodes * sizeof(BNode)));
  BNode* const d_nodes = *nodes_out;
  if (n == 1) {
    BNode nd;
    std::memset(&nd, 0, sizeof(nd));
    for (int a = 0; a < 3; ++a) {
      nd.c[0].lo[a] = hb[a];
      nd.c[0].hi[a] = hb[3 + a];
      nd.c[1].lo[a] = FLT_MAX;
      nd.c[1].hi[a] = -FLT_MAX;
    }
    uint32_t fl = 0;
    if (d_flags) HO_TRY(cudaMemcpy(&fl, d_flags, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    nd.c[0].idx = ~0;
    nd.c[0].aux = fl & kAuxHasField;
    nd.c[1].idx = kEmptyChild;
    HO_TRY(cudaMemcpy(d_nodes, &nd, sizeof(nd), cudaMemcpyHostToDevice));
    *depth_out = 1;
    return 0;
  }

  uint32_t *k0, *k1, *hist, *arrive;
  int32_t *v0, *v1, *pint, *pleaf;
  const int n_tiles = static_cast<int>((n + kSortTile - 1) / kSortTile);
  HO_TRY(cudaMalloc(&k0, n * sizeof(uint32_t)));
  HO_TRY(cudaMalloc(&k1, n * sizeof(uint32_t)));
  HO_TRY(cudaMalloc(&v0, n * sizeof(int32_t)));
  HO_TRY(cudaMalloc(&v1, n * sizeof(int32_t)));
  HO_TRY(cudaMalloc(&hist, static_cast<size_t>(256) * n_tiles * sizeof(uint32_t)));
  HO_TRY(cudaMalloc(&pint, n * sizeof(int32_t)));
  HO_TRY(cudaMalloc(&pleaf, n * sizeof(int32_t)));
  HO_TRY(cudaMalloc(&arrive, n * sizeof(uint32_t)));
  const unsigned gb = static_cast<unsigned>((n + 255) / 256);
  morton_kernel<<<gb, 256, 0, s>>>(d_box, n, lo, inv, k0, v0);
  HO_TRY(cudaGetLastError());
  for (int pass = 0; pass < 4; ++pass) {
    const int shift = 8 * pass;
    radix_hist_kernel<<<n_tiles, kSortTile, 0, s>>>(k0, n, shift, n_tiles, hist);
    scan_kernel<<<1, 1024, 0, s>>>(hist, static_cast<int64_t>(256) * n_tiles);
    radix_scatter_kernel<<<n_tiles, kSortTile, 0, s>>>(k0, v0, n, shift, n_tiles, hist, k1, v1);
    HO_TRY(cudaGetLastError());
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  HO_TRY(cudaMemsetAsync(pint, 0xff, n * sizeof(int32_t), s));
  HO_TRY(cudaMemsetAsync(arrive, 0, n * sizeof(uint32_t), s));
  karras_kernel<<<gb, 256, 0, s>>>(k0, v0, d_flags, n, d_nodes, pint, pleaf);
  HO_TRY(cudaGetLastError());
  refit_kernel<<<gb, 256, 0, s>>>(d_box, v0, n, d_nodes, pint, pleaf, arrive);
  HO_TRY(cudaGetLastError());

  // depth (host walk; also checks every node is reachable exactly once)
  std::vector<BNode> hn(n_nodes);
  HO_TRY(cudaMemcpyAsync(hn.data(), d_nodes, hn.size() * sizeof(BNode), cudaMemcpyDeviceToHost, s));
  HO_TRY(cudaStreamSynchronize(s));
  int depth = 0;
  int64_t leaves = 0;
  std::vector<std::pair<int32_t, int>> st;
  st.push_back({0, 1});
  int64_t visits = 0;
  while (!st.empty()) {
    if (++visits > n_nodes) break;  // a well-formed tree has exactly n_nodes internal nodes
    auto [id, dd] = st.back();
    st.pop_back();
    if (id < 0 || id >= n_nodes) break;
    depth = std::max(depth, dd);
    for (int ch = 0; ch < 2; ++ch) {
      const int32_t x = hn[id].c[ch].idx;
      if (x == kEmptyChild) continue;
      if (x < 0) ++leaves;
      else st.push_back({x, dd + 1});
    }
  }
  *depth_out = depth;
  cudaFree(k0);
  cudaFree(k1);
  cudaFree(v0);
  cudaFree(v1);
  cudaFree(hist);
  cudaFree(pint);
  cudaFree(pleaf);
  cudaFree(arrive);
  if (leaves != n) return int(cudaErrorUnknown);
  return 0;
}

}  // namespace ho
