// Host side of the element-major intersection rounds (batched and learned
// modes) and the small kernels between rounds: gather each ray's next
// candidate, bucket the pairs by element (counting sort), cut the buckets
// into batches, and write the final results.
#include <cuda_runtime.h>

#include <algorithm>

#include "ho_check.cuh"
#include "ho_host.h"
#include "ho_rounds.cuh"

namespace ho {

// Exclusive scan of the per-element pair counts in two launches over tiles of
// kScanTile values (1024 threads, 4 consecutive values each): the tiles'
// sums, then every tile's scan from its offset (the sum of the tiles before
// it, which each block adds up itself). One block carrying a running total
// through all the tiles takes time linear in the tile count (0.12 ms per
// round at 262,144 elements under a profiler; in the benchmark's graph the
// difference did not show).
constexpr int kScanTile = 4096;

__device__ __forceinline__ uint32_t block_sum_1024(uint32_t x, uint32_t* wsum) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
  if (lane == 0) wsum[wid] = x;
  __syncthreads();
  uint32_t t = lane < 32 ? wsum[lane] : 0u;
  if (wid == 0) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane == 0) wsum[0] = t;
  }
  __syncthreads();
  const uint32_t total = wsum[0];
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(1024) tile_sum_kernel(const uint32_t* __restrict__ in, int64_t len,
                                                        uint32_t* __restrict__ sums) {
  __shared__ uint32_t wsum[32];
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * 4;
  uint32_t t = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) t += i0 + k < len ? in[i0 + k] : 0u;
  const uint32_t total = block_sum_1024(t, wsum);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) tile_scan_kernel(const uint32_t* __restrict__ in, int64_t len,
                                                         const uint32_t* __restrict__ sums, uint32_t* __restrict__ out) {
  __shared__ uint32_t wsum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // this tile's offset: the sums of the tiles before it
  uint32_t pre = 0;
  for (unsigned b = threadIdx.x; b < blockIdx.x; b += blockDim.x) pre += sums[b];
  const uint32_t offset = block_sum_1024(pre, wsum);
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * kScanTile + static_cast<int64_t>(threadIdx.x) * 4;
  uint32_t v[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = i0 + k < len ? in[i0 + k] : 0u;
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
  uint32_t run = offset + (wid > 0 ? wsum[wid - 1] : 0u) + (x - t);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (i0 + k < len) out[i0 + k] = run;
    run += v[k];
  }
}

__global__ void round_init_kernel(RayState* __restrict__ st, const uint8_t* __restrict__ kovf,
                                  const unsigned* __restrict__ qcount) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *qcount) return;
  RayState r;
  r.best = miss_state();
  r.tie = miss_state();
  r.cursor = 0;
  r.pass = 0;
  r.kt = -FLT_MAX;
  r.ke = -1;
  r.done = 0;
  r.ovf = kovf[i];
  r.its = 0;
  r.pad = 0;
  st[i] = r;
}

// One thread per ray in flight: its next ordered candidate whose padded box
// the ray meets before the closest hit so far (the candidate loop of the
// reference's traversal, FEM-AABB/raytracer.cu:117-356, in ascending
// (entry t, element) order). A ray whose list was cut at kCandK walks the
// tree again for the candidates after the last visited one.
__global__ void round_gather_kernel(TraceParams P, RayState* __restrict__ st, RoundPair* __restrict__ pairs,
                                    int32_t* __restrict__ pelem, uint32_t* __restrict__ prank,
                                    uint32_t* __restrict__ ecount, unsigned* __restrict__ ctr) {
  const unsigned item = blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= *P.qcount) return;
  RayState& r = st[item];
  if (r.done) return;
  float3 o, d;
  float iso;
  bool iso_on;
  query_ray(P, P.work[item], o, d, iso, iso_on);
  Work w;
  float2* kb = P.kbuf + static_cast<int64_t>(item) * kCandK;
  for (int guard = 0; guard < (1 << 20); ++guard) {
    if (r.cursor >= kCandK) {
      if (!r.ovf) {
        r.done = 1;
        break;
      }
      float bt[kCandK];
      int be[kCandK];
      bool overflow;
      if (!collect(P, o, d, r.best.t, r.kt, r.ke, bt, be, overflow, w)) {
        atomicOr(&P.stats->status, kStatusStackOverflow);
        r.best.flags |= HO_FLAG_INCOMPLETE;
        r.done = 1;
        break;
      }
      for (int j = 0; j < kCandK; ++j) kb[j] = make_float2(bt[j], __int_as_float(be[j]));
      r.ovf = overflow ? 1 : 0;
      r.cursor = 0;
      ++r.pass;
      ++w.restarts;
      r.best.flags |= HO_FLAG_OVERFLOW;
    }
    const float2 c = kb[r.cursor];
    const float ct = c.x;
    const int ce = __float_as_int(c.y);
    if (ce == INT_MAX || ct > r.best.t) {
      r.done = 1;
      break;
    }
    const int j = r.cursor;
    ++r.cursor;
    r.kt = ct;
    r.ke = ce;
    const float* b = P.box + 6 * static_cast<int64_t>(ce);
    const float lo[3] = {__ldg(b), __ldg(b + 1), __ldg(b + 2)};
    const float hi[3] = {__ldg(b + 3), __ldg(b + 4), __ldg(b + 5)};
    float te, tx;
    if (!ray_box(o, d, lo, hi, 0.001f, r.best.t, te, tx)) continue;
    const unsigned k = atomicAdd(ctr, 1u);
    RoundPair p;
    p.item = static_cast<int32_t>(item);
    p.j = r.pass == 0 ? j : -1;
    p.te = te;
    p.tx = tx;
    pairs[k] = p;
    pelem[k] = ce;
    prank[k] = atomicAdd(&ecount[ce], 1u);
    break;
  }
  if (w.nodes || w.restarts) {
    atomicAdd(&P.stats->c[ST_NODES], static_cast<unsigned long long>(w.nodes));
    atomicAdd(&P.stats->c[ST_RESTART], static_cast<unsigned long long>(w.restarts));
  }
}

// Queued rays listed by a predicate (warp-aggregated appends): hits = false,
// the rays still in flight after the main rounds (for the tail kernel; the
// count goes to the work counters too); hits = true, the rays with a hit
// (for the FP64 check).
__global__ void ray_list_kernel(const unsigned* __restrict__ qcount, const RayState* __restrict__ st, bool hits,
                                uint32_t* __restrict__ list, unsigned* __restrict__ n_list, DevStats* stats) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  bool live = false;
  if (i < *qcount) live = hits ? st[i].best.kind != HO_HIT_MISS : !st[i].done;
  const unsigned m = __ballot_sync(kFull, live);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  unsigned base = 0;
  if (lane == leader) {
    base = atomicAdd(n_list, static_cast<unsigned>(__popc(m)));
    if (!hits) atomicAdd(&stats->c[ST_TAIL], static_cast<unsigned long long>(__popc(m)));
  }
  base = __shfl_sync(kFull, base, leader);
  if (live) list[base + __popc(m & ((1u << lane) - 1u))] = i;
}

// Also tallies the round (non-empty rounds and pairs) into the work counters.
__global__ void round_scatter_kernel(const RoundPair* __restrict__ pairs, const int32_t* __restrict__ pelem,
                                     const uint32_t* __restrict__ prank, const uint32_t* __restrict__ eoff,
                                     const unsigned* __restrict__ ctr, RoundPair* __restrict__ sorted,
                                     DevStats* stats) {
  const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned n_pairs = *ctr;
  if (k == 0 && n_pairs > 0) {
    atomicAdd(&stats->c[ST_ROUNDS], 1ull);
    atomicAdd(&stats->c[ST_PAIRS], static_cast<unsigned long long>(n_pairs));
  }
  if (k >= n_pairs) return;
  sorted[eoff[pelem[k]] + prank[k]] = pairs[k];
}

// Ctr layout: [0] pairs of the round, [3] failed FP64 checks, [4..5] the
// tail's list count and cursor, [6..7] the check's list count and tie count,
// and per order n (2..9) the batch count, region start, write cursor and take
// cursor.
constexpr int kCtrOrderNb = 16, kCtrOrderOff = 26, kCtrOrderCur = 36, kCtrOrderNext = 46, kCtrWords = 64;

__device__ __forceinline__ int batch_size(int chunk, int order, bool tc) {
  return chunk > 0 ? chunk : round_batch_default(order, tc);
}

// Batches per order: each element's pairs in batches of its order's size.
__global__ void round_batch_count_kernel(const uint32_t* __restrict__ ecount, const uint8_t* __restrict__ order,
                                         int64_t n_elem, int chunk, bool tc, unsigned* __restrict__ ctr) {
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  const int c = static_cast<int>(ecount[e]);
  if (c == 0) return;
  const int n = order[e];
  const int B = batch_size(chunk, n, tc);
  atomicAdd(&ctr[kCtrOrderNb + n], static_cast<unsigned>((c + B - 1) / B));
}

// Region start of each order's batches (orders in increasing n).
__global__ void round_order_offsets_kernel(unsigned* __restrict__ ctr) {
  unsigned run = 0;
  for (int n = 0; n < 10; ++n) {
    ctr[kCtrOrderOff + n] = run;
    ctr[kCtrOrderCur + n] = 0;
    ctr[kCtrOrderNext + n] = 0;
    run += ctr[kCtrOrderNb + n];
  }
}

// Each element's pairs in batches, written into its order's region.
__global__ void round_batch_kernel(const uint32_t* __restrict__ ecount, const uint32_t* __restrict__ eoff,
                                   const uint8_t* __restrict__ order, int64_t n_elem, int chunk, bool tc,
                                   RoundBatch* __restrict__ batches, unsigned* __restrict__ ctr) {
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n_elem) return;
  const int c = static_cast<int>(ecount[e]);
  if (c == 0) return;
  const int n = order[e];
  const int B = batch_size(chunk, n, tc);
  const int nb = (c + B - 1) / B;
  const unsigned base = ctr[kCtrOrderOff + n] + atomicAdd(&ctr[kCtrOrderCur + n], static_cast<unsigned>(nb));
  for (int k = 0; k < nb; ++k) {
    RoundBatch bt;
    bt.elem = static_cast<int32_t>(e);
    bt.first = static_cast<int32_t>(eoff[e]) + k * B;
    bt.count = min(B, c - k * B);
    bt.pad = 0;
    batches[base + k] = bt;
  }
}

// The queued rays' answers into the call's outputs; count: tally the grazing
// hits (once per call: a second write-out after extra rounds does not).
__global__ void round_finish_kernel(TraceParams P, const RayState* __restrict__ st, bool count) {
  const unsigned item = blockIdx.x * blockDim.x + threadIdx.x;
  if (item >= *P.qcount) return;
  const int64_t q = P.work[item];
  float3 o, d;
  float iso;
  bool iso_on;
  query_ray(P, q, o, d, iso, iso_on);
  const HitState& b = st[item].best;
  write_result(P, q, d, b, static_cast<uint32_t>(st[item].its));
  if (count) {
    const unsigned act = __activemask();
    const unsigned g = __ballot_sync(act, is_grazing(b, d));
    if (g && static_cast<int>(threadIdx.x & 31) == __ffs(act) - 1)
      atomicAdd(&P.stats->c[ST_GRAZING], static_cast<unsigned long long>(__popc(g)));
  }
}

// Grow-only device buffer of `want` elements of `size` bytes.
template <typename T>
static cudaError_t grow(T*& p, size_t& cap, size_t want, size_t size) {
  if (p && cap >= want) return cudaSuccess;
  cudaFree(p);
  p = nullptr;
  cap = 0;
  void* q = nullptr;
  const cudaError_t e = cudaMalloc(&q, std::max<size_t>(want, 1) * size);
  if (e == cudaSuccess) {
    p = static_cast<T*>(q);
    cap = want;
  }
  return e;
}

#define RT_TRY(x)                        \
  do {                                   \
    const cudaError_t e_ = (x);          \
    if (e_ != cudaSuccess) return int(e_); \
  } while (0)

// Scratch for up to n_cap queued rays (all queries of the call), allocated
// before any stream capture.
int prepare_rounds(ho_context* c, int64_t n_cap) {
  const size_t n = static_cast<size_t>(std::max<int64_t>(n_cap, 1));
  const int64_t n_elem = c->n_elem;
  RoundBufs& rb = c->rounds;
  RT_TRY(grow(rb.state, rb.state_cap, n, sizeof(RayState)));
  RT_TRY(grow(rb.pairs, rb.pairs_cap, 2 * n, sizeof(RoundPair)));
  RT_TRY(grow(rb.pelem, rb.pelem_cap, n, sizeof(int32_t)));
  RT_TRY(grow(rb.prank, rb.prank_cap, n, sizeof(uint32_t)));
  RT_TRY(grow(rb.batches, rb.batches_cap, n, sizeof(RoundBatch)));
  RT_TRY(grow(rb.ecount, rb.ecount_cap, static_cast<size_t>(n_elem), sizeof(uint32_t)));
  RT_TRY(grow(rb.eoff, rb.eoff_cap, static_cast<size_t>(n_elem), sizeof(uint32_t)));
  RT_TRY(grow(rb.tile_sums, rb.tile_sums_cap, static_cast<size_t>((n_elem + kScanTile - 1) / kScanTile),
              sizeof(uint32_t)));
  RT_TRY(grow(rb.ctr, rb.ctr_cap, kCtrWords, sizeof(unsigned)));
  RT_TRY(grow(rb.fail, rb.fail_cap, n, sizeof(uint32_t)));
  return 0;
}

// The check's residuals for caller-given hits (ho_hit_residuals).
int launch_residuals(ho_context* c, int64_t n, const float* rays, const ho_hit* hits, double* out, cudaStream_t s) {
  cudaError_t e;
  switch (c->N) {
    case 2: e = launch_residuals_n<2>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    case 3: e = launch_residuals_n<3>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    case 4: e = launch_residuals_n<4>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    case 5: e = launch_residuals_n<5>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    case 6: e = launch_residuals_n<6>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    case 7: e = launch_residuals_n<7>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    case 8: e = launch_residuals_n<8>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    case 9: e = launch_residuals_n<9>(c->d_rec, c->d_flags, n, rays, hits, out, s); break;
    default: e = cudaErrorInvalidValue; break;
  }
  return int(e);
}

// FP64 check of the rays' hits, plain fallback of the failures.
static int enqueue_check(ho_context* c, const TraceParams& P, const RoundParams& R, cudaStream_t s, int64_t n_cap) {
  if (!c->fp64_check) return 0;
  // the rays with a hit, listed into the (now idle) pair-element buffer, so
  // that the check's threads are all busy
  uint32_t* list = reinterpret_cast<uint32_t*>(c->rounds.pelem);
  unsigned* n_list = c->rounds.ctr + 6;
  unsigned* n_tie = c->rounds.ctr + 7;
  RT_TRY(cudaMemsetAsync(c->rounds.ctr + 3, 0, sizeof(unsigned), s));
  RT_TRY(cudaMemsetAsync(n_list, 0, 2 * sizeof(unsigned), s));
  ray_list_kernel<<<static_cast<unsigned>((n_cap + 255) / 256), 256, 0, s>>>(P.qcount, R.state, true, list, n_list,
                                                                             P.stats);
  RT_TRY(cudaGetLastError());
  c->launches += 4;  // ray list, check, tie rule, fallback
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e;
  switch (c->N) {
    case 2:
      e = launch_check_n<2>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    case 3:
      e = launch_check_n<3>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    case 4:
      e = launch_check_n<4>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    case 5:
      e = launch_check_n<5>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    case 6:
      e = launch_check_n<6>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    case 7:
      e = launch_check_n<7>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    case 8:
      e = launch_check_n<8>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    case 9:
      e = launch_check_n<9>(P, R.state, list, n_list, c->rounds.fail, c->rounds.ctr + 3, n_tie, n_cap, sms, s);
      break;
    default: e = cudaErrorInvalidValue; break;
  }
  RT_TRY(e);
  return 0;
}

static RoundParams round_params(ho_context* c, const TraceParams& P) {
  RoundBufs& rb = c->rounds;
  RoundParams R;
  R.rec = P.rec;
  R.fbox = P.fbox;
  R.flags = P.flags;
  R.rays = P.rays;
  R.n_rays = P.n_rays;
  R.cam = P.cam;
  for (int i = 0; i < 8; ++i) R.iso[i] = P.iso[i];
  R.iso_on_mask = P.iso_on_mask;
  R.views = P.views;
  R.n_views = P.n_views;
  R.work = P.work;
  R.state = static_cast<RayState*>(rb.state);
  R.pairs = static_cast<RoundPair*>(rb.pairs) + rb.pairs_cap / 2;
  R.batches = static_cast<RoundBatch*>(rb.batches);
  R.batch_base = rb.ctr + kCtrOrderOff + c->N;
  R.n_batches = rb.ctr + kCtrOrderNb + c->N;
  R.next_batch = rb.ctr + kCtrOrderNext + c->N;
  R.crec = c->d_crec;
  R.coff = c->d_coff;
  R.stats = P.stats;
  R.desc = P.desc;
  R.cand_e = P.cand_e;
  R.pred = P.pred;
  R.pred_items = P.pred_items;
  R.warm_cap = c->warm_cap;
  return R;
}

// Records an event on s; inside a stream capture the event becomes an event
// record node of the graph, so its time is taken when the graph runs.
static cudaError_t record_event(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cs);
  if (e != cudaSuccess) return e;
  return cudaEventRecordWithFlags(ev, s, cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                               : cudaEventRecordDefault);
}

// The next pair of timing events of this call (created on first use).
static cudaError_t next_events(ho_context* c, cudaEvent_t* a, cudaEvent_t* b) {
  while (static_cast<int>(c->round_events.size()) < c->round_events_used + 2) {
    cudaEvent_t ev = nullptr;
    const cudaError_t e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return e;
    c->round_events.push_back(ev);
  }
  *a = c->round_events[c->round_events_used];
  *b = c->round_events[c->round_events_used + 1];
  c->round_events_used += 2;
  return cudaSuccess;
}

// One round: gather each ray's next pair, bucket by element, intersect. Every
// launch has a fixed size and reads its counts on the device, so rounds can
// be enqueued (and captured) without reading anything back.
static int enqueue_round(ho_context* c, const TraceParams& P, const RoundParams& R, cudaStream_t s, bool learned,
                         int64_t n_cap) {
  RoundBufs& rb = c->rounds;
  const int64_t n_elem = c->n_elem;
  RoundPair* gathered = static_cast<RoundPair*>(rb.pairs);
  const unsigned gi = static_cast<unsigned>((n_cap + 255) / 256);
  RT_TRY(cudaMemsetAsync(rb.ecount, 0, static_cast<size_t>(n_elem) * sizeof(uint32_t), s));
  RT_TRY(cudaMemsetAsync(rb.ctr, 0, kCtrWords * sizeof(unsigned), s));
  round_gather_kernel<<<gi, 256, 0, s>>>(P, R.state, gathered, rb.pelem, rb.prank, rb.ecount, rb.ctr);
  {
    const unsigned tiles = static_cast<unsigned>((n_elem + kScanTile - 1) / kScanTile);
    if (tiles > 0) {
      tile_sum_kernel<<<tiles, 1024, 0, s>>>(rb.ecount, n_elem, rb.tile_sums);
      tile_scan_kernel<<<tiles, 1024, 0, s>>>(rb.ecount, n_elem, rb.tile_sums, rb.eoff);
    }
  }
  round_scatter_kernel<<<gi, 256, 0, s>>>(gathered, rb.pelem, rb.prank, rb.eoff, rb.ctr,
                                          const_cast<RoundPair*>(R.pairs), P.stats);
  const unsigned ge = static_cast<unsigned>((n_elem + 255) / 256);
  round_batch_count_kernel<<<ge, 256, 0, s>>>(rb.ecount, c->d_cord, n_elem, c->round_chunk, c->use_tc, rb.ctr);
  round_order_offsets_kernel<<<1, 1, 0, s>>>(rb.ctr);
  round_batch_kernel<<<ge, 256, 0, s>>>(rb.ecount, rb.eoff, c->d_cord, n_elem, c->round_chunk, c->use_tc,
                                        const_cast<RoundBatch*>(R.batches), rb.ctr);
  RT_TRY(cudaGetLastError());
  c->launches += 7 + __builtin_popcount(c->orders);
  // one launch per element order present in the scene
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (c->time_rounds) {
    RT_TRY(next_events(c, &t0, &t1));
    RT_TRY(record_event(t0, s));
  }
  cudaError_t e = cudaSuccess;
  for (int n = kMinModes; n <= kMaxModes && e == cudaSuccess; ++n) {
    if (!((c->orders >> n) & 1u)) continue;
    RoundParams Rn = R;
    Rn.batch_base = rb.ctr + kCtrOrderOff + n;
    Rn.n_batches = rb.ctr + kCtrOrderNb + n;
    Rn.next_batch = rb.ctr + kCtrOrderNext + n;
    switch (n) {
      case 2: e = launch_round_n<2>(Rn, s, learned, c->use_tc); break;
      case 3: e = launch_round_n<3>(Rn, s, learned, c->use_tc); break;
      case 4: e = launch_round_n<4>(Rn, s, learned, c->use_tc); break;
      case 5: e = launch_round_n<5>(Rn, s, learned, c->use_tc); break;
      case 6: e = launch_round_n<6>(Rn, s, learned, c->use_tc); break;
      case 7: e = launch_round_n<7>(Rn, s, learned, c->use_tc); break;
      case 8: e = launch_round_n<8>(Rn, s, learned, c->use_tc); break;
      case 9: e = launch_round_n<9>(Rn, s, learned, c->use_tc); break;
      default: e = cudaErrorInvalidValue; break;
    }
  }
  RT_TRY(e);
  if (t1) RT_TRY(record_event(t1, s));
  return 0;
}

// The tail: every ray still in flight finished by the warp-per-ray kernel;
// afterwards no round has pairs left (ctr[0] = 0).
static int enqueue_tail(ho_context* c, const TraceParams& P, const RoundParams& R, cudaStream_t s, bool learned,
                        int64_t n_cap) {
  RoundBufs& rb = c->rounds;
  unsigned* n_list = rb.ctr + 4;
  unsigned* next = rb.ctr + 5;
  RT_TRY(cudaMemsetAsync(rb.ctr + 4, 0, 2 * sizeof(unsigned), s));
  ray_list_kernel<<<static_cast<unsigned>((n_cap + 255) / 256), 256, 0, s>>>(P.qcount, R.state, false, rb.fail,
                                                                             n_list, P.stats);
  RT_TRY(cudaGetLastError());
  cudaError_t e;
  switch (c->N) {
    case 2: e = launch_tail_n<2>(P, R.state, rb.fail, n_list, next, learned, s); break;
    case 3: e = launch_tail_n<3>(P, R.state, rb.fail, n_list, next, learned, s); break;
    case 4: e = launch_tail_n<4>(P, R.state, rb.fail, n_list, next, learned, s); break;
    case 5: e = launch_tail_n<5>(P, R.state, rb.fail, n_list, next, learned, s); break;
    case 6: e = launch_tail_n<6>(P, R.state, rb.fail, n_list, next, learned, s); break;
    case 7: e = launch_tail_n<7>(P, R.state, rb.fail, n_list, next, learned, s); break;
    case 8: e = launch_tail_n<8>(P, R.state, rb.fail, n_list, next, learned, s); break;
    case 9: e = launch_tail_n<9>(P, R.state, rb.fail, n_list, next, learned, s); break;
    default: e = cudaErrorInvalidValue; break;
  }
  RT_TRY(e);
  RT_TRY(cudaMemsetAsync(rb.ctr, 0, sizeof(unsigned), s));
  c->launches += 2;
  return 0;
}

// The state init, `rounds` rounds (then the tail, when on) and the final
// write-out of the queued rays.
int enqueue_rounds(ho_context* c, const TraceParams& P, cudaStream_t s, bool learned, int64_t n_cap, int rounds) {
  const RoundParams R = round_params(c, P);
  const unsigned gi = static_cast<unsigned>((n_cap + 255) / 256);
  round_init_kernel<<<gi, 256, 0, s>>>(R.state, P.kovf, P.qcount);
  RT_TRY(cudaGetLastError());
  c->launches += 2;  // init and finish
  // with the tail, a fixed number of rounds (the tail finishes every ray)
  if (c->tail_after > 0) rounds = std::min(c->round_count, c->tail_after);
  for (int r = 0; r < rounds; ++r) {
    const int rc = enqueue_round(c, P, R, s, learned, n_cap);
    if (rc) return rc;
  }
  if (c->tail_after > 0) {
    const int rc = enqueue_tail(c, P, R, s, learned, n_cap);
    if (rc) return rc;
  }
  {
    const int rc = enqueue_check(c, P, R, s, n_cap);
    if (rc) return rc;
  }
  round_finish_kernel<<<gi, 256, 0, s>>>(P, R.state, true);
  RT_TRY(cudaGetLastError());
  return 0;
}

// After the enqueued rounds ran: while the last round still found pairs, run
// one more round (with a read-back each), then write the results again.
int finish_rounds(ho_context* c, const TraceParams& P, cudaStream_t s, bool learned, int64_t n_cap) {
  const RoundParams R = round_params(c, P);
  bool extra = false;
  for (int guard = 0; guard < 100000; ++guard) {
    unsigned last = 0;
    unsigned long long rounds = 0;
    RT_TRY(cudaMemcpyAsync(&last, c->rounds.ctr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    RT_TRY(cudaMemcpyAsync(&rounds, &P.stats->c[ST_ROUNDS], sizeof(rounds), cudaMemcpyDeviceToHost, s));
    RT_TRY(cudaStreamSynchronize(s));
    c->rounds_needed = static_cast<int>(rounds);
    if (last == 0) break;
    extra = true;
    const int rc = enqueue_round(c, P, R, s, learned, n_cap);
    if (rc) return rc;
  }
  if (extra) {
    const int rc = enqueue_check(c, P, R, s, n_cap);
    if (rc) return rc;
    round_finish_kernel<<<static_cast<unsigned>((n_cap + 255) / 256), 256, 0, s>>>(P, R.state, false);
    RT_TRY(cudaGetLastError());
    ++c->launches;
  }
  return 0;
}

}  // namespace ho
