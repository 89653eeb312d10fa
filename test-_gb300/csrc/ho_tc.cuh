// Tensor-core evaluation of an element's contractions for 128 points at once
// (tcgen05.mma kind::tf32, accumulators in tensor memory), used by the round
// kernel's tensor-core form.
//
// The first contraction of a component block, T[k][j](point) =
// sum_i c[k][j][i] a_i(xi1), is a GEMM over the element's coefficients:
// D[point][(comp,k,j)] = sum_i A[point][i] * B[(comp,k,j)][i], with K = 8
// (i < N, zero beyond) and one row of A per thread of the CTA. The derivative
// basis da_i(xi1) gives a second GEMM into a second accumulator. FP32 operands
// are split into TF32 hi + lo and the three significant products (lo*hi,
// hi*lo, hi*hi) are accumulated in FP32, about 2^-21 relative per product.
// The remaining contractions over j and k (3N^2 + 4N FMAs per component)
// run on the CUDA cores from the accumulator rows read back with tcgen05.ld:
// thread t of the CTA owns tensor-memory lane t, i.e. its own point's row.
//
// Layouts (K-major, no swizzle): both operands are stored as core matrices of
// 8 rows x 16 bytes (8 rows x 4 TF32); a row's 8 K values are two core
// matrices 128 bytes apart (leading byte offset), consecutive 8-row groups
// are 256 bytes apart (stride byte offset).
#pragma once

#include <cstdint>

namespace ho {

constexpr int kTcRows = 128;        // MMA M: one point per thread of the CTA
constexpr int kTcCompCols = 64;     // accumulator columns per component (N*N <= 64)
constexpr int kTcCols = 4 * kTcCompCols;  // MMA N: x, y, z, field
constexpr int kTcTmemCols = 2 * kTcCols;  // value and derivative accumulators
constexpr int kTcLbo = 128, kTcSbo = 256;

// Float offset of element (row r, k) in a K-major 8-wide operand tile.
__host__ __device__ constexpr int tc_core_off(int r, int k) {
  return (r >> 3) * 64 + (k >> 2) * 32 + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, leading / stride byte
// offsets (16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((kTcLbo >> 4) & 0x3FFF) << 16) |
         (static_cast<uint64_t>((kTcSbo >> 4) & 0x3FFF) << 32) | (static_cast<uint64_t>(1) << 46);
}

// Instruction descriptor: D f32, A and B tf32, both K-major, N = kTcCols, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((static_cast<uint32_t>(kTcCols) >> 3) << 17) |
                              ((static_cast<uint32_t>(kTcRows) >> 4) << 24);

// TF32 value nearest to x (round to nearest, ties away), as an FP32 bit pattern.
__device__ __forceinline__ float tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void tc_alloc(uint32_t* slot) {  // one warp
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(slot)),
               "n"(kTcTmemCols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr) {  // the same warp
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "n"(kTcTmemCols));
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t da, uint64_t db, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(da), "l"(db), "r"(kTcIdesc), "r"(accumulate ? 1 : 0));
}

__device__ __forceinline__ void tc_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   tc_smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void tc_mbar_init(uint64_t* mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem_u32(mbar)));
  asm volatile("fence.mbarrier_init.release.cluster;");
}

// Waits for the phase with the given parity to complete; false after the
// iteration limit.
__device__ __forceinline__ bool tc_mbar_wait(uint64_t* mbar, uint32_t parity) {
  const uint32_t a = tc_smem_u32(mbar);
  for (int it = 0; it < (1 << 24); ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16 consecutive accumulator columns of this warp's 32 lanes (one per thread).
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// Shared memory of the tensor-core evaluation: the element's coefficients as
// the B operand (hi and lo parts) and the four A operand tiles of the step.
struct TcSm {
  float bhi[kTcCols * 8];
  float blo[kTcCols * 8];
  float a[4][kTcRows * 8];  // basis hi, basis lo, derivative hi, derivative lo
  uint64_t mbar;
  uint32_t tslot;
  unsigned ctl[4];  // round kernel: [0] batch, [1] pairs claimed, [2] spare
};

// The element's coefficient record (rows padded to row_stride(N)) as the B
// operand: row (comp, k*N + j) of the GEMM holds c[comp][k][j][0..N), zeros
// beyond. Every thread of the CTA takes a share.
template <int N>
__device__ __forceinline__ void tc_stage_b(TcSm& T, const float* __restrict__ rec, int tid, int nthreads) {
  constexpr int RS = row_stride(N);
  for (int e = tid; e < kTcCols * 8; e += nthreads) {
    const int n = e >> 3, i = e & 7;
    const int comp = n / kTcCompCols, kj = n % kTcCompCols;
    float x = 0.f;
    if (kj < N * N && i < N) x = __ldg(rec + comp * block_floats(N) + kj * RS + i);
    const float hi = tc_tf32(x);
    T.bhi[tc_core_off(n, i)] = hi;
    T.blo[tc_core_off(n, i)] = tc_tf32(x - hi);
  }
}

// This thread's A rows: the xi1 basis values and derivatives, split.
template <int N>
__device__ __forceinline__ void tc_stage_a(TcSm& T, int row, const float (&ar)[N], const float (&dr)[N]) {
  float v[4][8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float a = i < N ? ar[i] : 0.f, d = i < N ? dr[i] : 0.f;
    const float ah = tc_tf32(a), dh = tc_tf32(d);
    v[0][i] = ah;
    v[1][i] = tc_tf32(a - ah);
    v[2][i] = dh;
    v[3][i] = tc_tf32(d - dh);
  }
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    float4* lo4 = reinterpret_cast<float4*>(&T.a[m][tc_core_off(row, 0)]);
    float4* hi4 = reinterpret_cast<float4*>(&T.a[m][tc_core_off(row, 4)]);
    *lo4 = make_float4(v[m][0], v[m][1], v[m][2], v[m][3]);
    *hi4 = make_float4(v[m][4], v[m][5], v[m][6], v[m][7]);
  }
}

// One thread issues the six MMAs of a step and commits them to the barrier:
// value accumulator at column 0, derivative accumulator at kTcCols; small
// products first.
__device__ __forceinline__ void tc_issue(TcSm& T, uint32_t tmem) {
  const uint64_t bh = tc_desc(tc_smem_u32(T.bhi)), bl = tc_desc(tc_smem_u32(T.blo));
  const uint64_t ah = tc_desc(tc_smem_u32(T.a[0])), al = tc_desc(tc_smem_u32(T.a[1]));
  const uint64_t dh = tc_desc(tc_smem_u32(T.a[2])), dl = tc_desc(tc_smem_u32(T.a[3]));
  tc_mma(tmem, al, bh, false);
  tc_mma(tmem, ah, bl, true);
  tc_mma(tmem, ah, bh, true);
  tc_mma(tmem + kTcCols, dl, bh, false);
  tc_mma(tmem + kTcCols, dh, bl, true);
  tc_mma(tmem + kTcCols, dh, bh, true);
  tc_commit(&T.mbar);
}

// The rest of component comp for this thread's point from its accumulator row
// (taddr = the warp's lane base): value and the three partials. Every lane of
// the warp must call it (tcgen05.ld is warp-wide).
template <int N>
__device__ __forceinline__ float4 tc_finish_comp(uint32_t taddr, int comp, const float (&as)[N], const float (&ds)[N],
                                                 const float (&at)[N], const float (&dt)[N]) {
  constexpr int NN = N * N;
  constexpr int NCH = (NN + 15) / 16;
  float qa[N], qs[N], qd[N];
#pragma unroll
  for (int k = 0; k < N; ++k) qa[k] = qs[k] = qd[k] = 0.f;
#pragma unroll
  for (int ch = 0; ch < NCH; ++ch) {
    float ta[16], td[16];
    tc_ld16(taddr + comp * kTcCompCols + ch * 16, ta);
    tc_ld16(taddr + kTcCols + comp * kTcCompCols + ch * 16, td);
    tc_wait_ld();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int n = ch * 16 + q;
      if (n < NN) {
        const int k = n / N, j = n % N;
        qa[k] = fmaf(ta[q], as[j], qa[k]);
        qs[k] = fmaf(ta[q], ds[j], qs[k]);
        qd[k] = fmaf(td[q], as[j], qd[k]);
      }
    }
  }
  float v = 0.f, vr = 0.f, vs = 0.f, vt = 0.f;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    v = fmaf(qa[k], at[k], v);
    vr = fmaf(qd[k], at[k], vr);
    vs = fmaf(qs[k], at[k], vs);
    vt = fmaf(qa[k], dt[k], vt);
  }
  return make_float4(v, vr, vs, vt);
}

}  // namespace ho
