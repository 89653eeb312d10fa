// Dispatch of the trace kernel by modes per direction; each instantiation
// lives in its own translation unit (ho_trace_n*.cu) so they compile in
// parallel.
#include <algorithm>

#include "ho_mlp_infer.cuh"
#include "ho_trace.cuh"

namespace ho {

// Pass 1, one thread per query: rays that meet no padded box are finished
// here (miss); the rest are appended to the work queue together with their
// first kCandK ordered candidates.
__global__ void __launch_bounds__(256) classify_kernel(TraceParams P, int64_t n_queries) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  Work w;
  bool need = false, overflow = false, incomplete = false;
  float bt[kCandK];
  int be[kCandK];
  float3 o = make_float3(0.f, 0.f, 0.f), d = make_float3(0.f, 0.f, 1.f);
  if (q < n_queries) {
    float iso;
    bool iso_on;
    query_ray(P, q, o, d, iso, iso_on);
    // the ray's first kCandK ordered candidates (nothing is hit yet, so the
    // bound is infinite): the intersect pass starts from this list
    if (!collect(P, o, d, FLT_MAX, -FLT_MAX, -1, bt, be, overflow, w)) {
      atomicOr(&P.stats->status, kStatusStackOverflow);
      be[0] = INT_MAX;
      incomplete = true;
    }
    need = be[0] != INT_MAX;
    if (!need) {
      HitState m = miss_state();
      if (incomplete) m.flags |= HO_FLAG_INCOMPLETE;
      write_result(P, q, d, m, 0);
    }
  }
  const unsigned m = __ballot_sync(kFull, need);
  if (m) {
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(P.qcount, static_cast<unsigned>(__popc(m)));
    base = __shfl_sync(kFull, base, leader);
    if (need) {
      const unsigned slot = base + __popc(m & ((1u << lane) - 1u));
      P.work[slot] = static_cast<int32_t>(q);
      float2* kb = P.kbuf + static_cast<int64_t>(slot) * kCandK;
#pragma unroll
      for (int j = 0; j < kCandK; ++j) kb[j] = make_float2(bt[j], __int_as_float(be[j]));
      P.kovf[slot] = overflow ? 1 : 0;
    }
  }
  flush_work(P.stats, w, q < n_queries);
}

// Learned mode, after classify: the network's predictions for the first
// kPredK ordered candidates of each queued ray (the same as the rounds' first
// candidates: nothing is hit yet). The input row of a (ray, candidate) pair
// is formed in the kernel that runs the network, two lanes per row, from the
// candidate list, the element's descriptor and the ray (the same values as
// write_features); its element goes to cand_e (-1: no candidate, zero row).
struct CandRows {
  const TraceParams& P;
  int32_t* cand_e;
  __device__ __forceinline__ void fill(int64_t row, int half, __nv_bfloat16* dst) const {
    const int64_t item = row / kPredK;
    const int j = static_cast<int>(row % kPredK);
    const float2 c = P.kbuf[item * kCandK + j];
    const int ce = __float_as_int(c.y);
    const int e = ce != INT_MAX ? ce : -1;
    if (half == 0) cand_e[row] = e;
    __nv_bfloat162* d2 = reinterpret_cast<__nv_bfloat162*>(dst);
    if (e < 0) {
      const __nv_bfloat162 z = __floats2bfloat162_rn(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < kMlpInPad / 4; ++q) d2[q] = z;
      return;
    }
    const float* desc = P.desc + static_cast<int64_t>(e) * kDescFloats;
    if (half == 0) {  // columns 0..31: descriptor values
#pragma unroll
      for (int q = 0; q < 16; ++q) d2[q] = __floats2bfloat162_rn(__ldg(desc + 2 * q), __ldg(desc + 2 * q + 1));
      return;
    }
    // columns 32..63: descriptor 32..41, entry point, direction, zero pad
#pragma unroll
    for (int q = 0; q < 5; ++q) d2[q] = __floats2bfloat162_rn(__ldg(desc + 32 + 2 * q), __ldg(desc + 33 + 2 * q));
    float3 o, d;
    float iso;
    bool iso_on;
    query_ray(P, P.work[item], o, d, iso, iso_on);
    float f[6];
    feature_tail(desc, o, d, c.x, f);
    d2[5] = __floats2bfloat162_rn(f[0], f[1]);
    d2[6] = __floats2bfloat162_rn(f[2], f[3]);
    d2[7] = __floats2bfloat162_rn(f[4], f[5]);
    const __nv_bfloat162 z = __floats2bfloat162_rn(0.f, 0.f);
#pragma unroll
    for (int q = 8; q < 16; ++q) d2[q] = z;
  }
};

__global__ void __launch_bounds__(256) pred_kernel(MlpDev M, TraceParams P, int32_t* __restrict__ cand_e,
                                                   float* __restrict__ Y) {
  // predictions for the first pred_items queued rays (the buffers' size); the
  // rest start cold
  const unsigned n_work = min(*P.qcount, P.pred_items);
  if (blockIdx.x == 0 && threadIdx.x == 0) P.qcount[2] = n_work;
  mlp_infer_tiles(M, CandRows{P, cand_e}, static_cast<int64_t>(n_work) * kPredK, Y);
}

static int launch_pred(ho_context* c, const TraceParams& P, cudaStream_t s, int sms) {
  // the attribute is set once per device
  static std::atomic<bool> attr[kGridCacheDevices];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return int(e);
  if (dev < 0 || dev >= kGridCacheDevices) return int(cudaErrorInvalidDevice);
  if (!attr[dev].load(std::memory_order_acquire)) {
    e = cudaFuncSetAttribute(pred_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(sizeof(InferSmem)));
    if (e != cudaSuccess) return int(e);
    attr[dev].store(true, std::memory_order_release);
  }
  pred_kernel<<<sms, 256, sizeof(InferSmem), s>>>(c->mlp.dev(), P, c->d_cand, c->d_pred);
  return int(cudaGetLastError());
}

int prepare_rounds(ho_context* c, int64_t n_cap);
int enqueue_rounds(ho_context* c, const TraceParams& P, cudaStream_t s, bool learned, int64_t n_cap, int rounds);
int finish_rounds(ho_context* c, const TraceParams& P, cudaStream_t s, bool learned, int64_t n_cap);

// Everything of a batched / learned call that runs on the stream: the
// classify pass, the network (learned), the rounds and the write-out. No host
// read-back and no allocation, so the whole sequence can be captured.
static int enqueue_batched(ho_context* c, TraceParams& P, cudaStream_t s, bool learned, int64_t n_queries, int sms) {
  cudaError_t e = cudaMemsetAsync(c->d_qctr, 0, 4 * sizeof(unsigned), s);
  if (e != cudaSuccess) return int(e);
  classify_kernel<<<static_cast<unsigned>((n_queries + 255) / 256), 256, 0, s>>>(P, n_queries);
  e = cudaGetLastError();
  if (e != cudaSuccess) return int(e);
  ++c->launches;
  if (learned) {
    ++c->launches;
    const int rc = launch_pred(c, P, s, sms);
    if (rc) return rc;
  }
  // as many rounds as the previous call needed, plus one, within the option
  const int rounds = c->rounds_needed > 0 ? std::min(c->round_count, c->rounds_needed + 1) : c->round_count;
  return enqueue_rounds(c, P, s, learned, n_queries, rounds);
}

static int trace_hexes(ho_context* c, const TraceArgs& a, cudaStream_t s) {
  c->last_graph = false;
  c->stats_frozen = false;
  c->launches = 0;
  c->round_events_used = 0;
  TraceParams P;
  P.nodes = c->d_nodes;
  P.rec = c->d_rec;
  P.fbox = c->d_fbox;
  P.box = c->d_box;
  P.flags = c->d_flags;
  P.rays = a.rays;
  P.n_rays = a.n_rays;
  P.cam = cam_args(a);
  for (int i = 0; i < 8; ++i) P.iso[i] = i < a.n_iso ? a.iso[i] : 0.f;
  P.n_iso = a.n_iso;
  P.iso_on_mask = a.iso_on_mask;
  P.views = a.views;
  P.n_views = a.n_views;
  P.hits = a.hits;
  P.rgb = a.rgb;
  P.stats = c->d_stats;
  P.fp64 = c->fp64_check ? 1 : 0;
  int64_t n_queries, n_threads;
  if (a.rays) {
    n_queries = a.n_rays * a.n_iso;
    n_threads = n_queries;
  } else if (a.views) {
    n_queries = a.n_queries_views;
    n_threads = n_queries;
  } else {
    const int64_t tiles = static_cast<int64_t>((a.width + 7) / 8) * ((a.height + 3) / 4);
    n_queries = static_cast<int64_t>(a.width) * a.height * a.n_iso;
    n_threads = tiles * 32 * a.n_iso;
  }
  if (n_threads == 0) return 0;
  if (static_cast<size_t>(n_queries) > c->work_cap || !c->d_work) {
    cudaFree(c->d_work);
    cudaFree(c->d_kbuf);
    cudaFree(c->d_kovf);
    c->d_work = nullptr;
    c->d_kbuf = nullptr;
    c->d_kovf = nullptr;
    c->work_cap = 0;
    cudaError_t e = cudaMalloc(&c->d_work, static_cast<size_t>(n_queries) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_kbuf, static_cast<size_t>(n_queries) * kCandK * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_kovf, static_cast<size_t>(n_queries));
    if (e != cudaSuccess) return int(e);
    c->work_cap = static_cast<size_t>(n_queries);
  }
  if (!c->d_qctr) {
    cudaError_t e = cudaMalloc(&c->d_qctr, 4 * sizeof(unsigned));
    if (e != cudaSuccess) return int(e);
  }
  {
    cudaError_t e = cudaMemsetAsync(c->d_qctr, 0, 4 * sizeof(unsigned), s);
    if (e != cudaSuccess) return int(e);
  }
  const int mode = (c->mode == HO_MODE_LEARNED && !c->mlp.trained) ? HO_MODE_BATCHED : c->mode;
  if (mode == HO_MODE_PLAIN) {
    // one thread per query: camera queries are laid out as 8x4 pixel tiles per warp
    if (!a.rays && !a.views) n_threads = static_cast<int64_t>((a.width + 7) / 8) * ((a.height + 3) / 4) * 32 * a.n_iso;
    cudaError_t e;
    switch (c->N) {
      case 2: e = launch_n<2>(P, n_queries, n_threads, s, mode); break;
      case 3: e = launch_n<3>(P, n_queries, n_threads, s, mode); break;
      case 4: e = launch_n<4>(P, n_queries, n_threads, s, mode); break;
      case 5: e = launch_n<5>(P, n_queries, n_threads, s, mode); break;
      case 6: e = launch_n<6>(P, n_queries, n_threads, s, mode); break;
      case 7: e = launch_n<7>(P, n_queries, n_threads, s, mode); break;
      case 8: e = launch_n<8>(P, n_queries, n_threads, s, mode); break;
      case 9: e = launch_n<9>(P, n_queries, n_threads, s, mode); break;
      default: return int(cudaErrorInvalidValue);
    }
    c->launches = 1;
    return int(e);
  }
  P.work = c->d_work;
  P.qcount = c->d_qctr;
  P.qnext = c->d_qctr + 1;
  P.kbuf = c->d_kbuf;
  P.kovf = c->d_kovf;
  const bool learned = mode == HO_MODE_LEARNED;
  // allocate first: nothing enqueued below may allocate (it may be captured)
  P.pred_items = static_cast<unsigned>(std::min<int64_t>(n_queries, kPredItemsCap));
  if (learned) {
    const size_t rows = static_cast<size_t>(P.pred_items) * kPredK;
    if (rows > c->pred_cap) {
      cudaFree(c->d_pred);
      cudaFree(c->d_cand);
      c->d_pred = nullptr;
      c->d_cand = nullptr;
      c->pred_cap = 0;
      cudaError_t e = cudaMalloc(&c->d_pred, rows * kMlpOut * sizeof(float));
      if (e == cudaSuccess) e = cudaMalloc(&c->d_cand, rows * sizeof(int32_t));
      if (e != cudaSuccess) return int(e);
      c->pred_cap = rows;
    }
  }
  {
    const int rc = prepare_rounds(c, n_queries);
    if (rc) return rc;
  }
  P.desc = c->d_desc;
  P.cand_e = learned ? c->d_cand : nullptr;
  P.pred = learned ? c->d_pred : nullptr;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);

  // The first call of a context runs its launches directly (first-use set-up
  // of kernel attributes happens there); later calls are captured into one
  // CUDA graph, whose executable is patched in place while the launch
  // sequence keeps its shape.
  bool capture = c->use_graph && c->graph_warm;
  if (capture && cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    capture = false;
  }
  int rc = enqueue_batched(c, P, s, learned, n_queries, sms);
  if (capture) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc == 0 && e != cudaSuccess) rc = int(e);
    if (rc == 0 && c->graph_exec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(c->graph_exec, g, &info) != cudaSuccess) {
        cudaGetLastError();
        cudaGraphExecDestroy(c->graph_exec);
        c->graph_exec = nullptr;
      }
    }
    if (rc == 0 && !c->graph_exec) {
      e = cudaGraphInstantiate(&c->graph_exec, g, 0);
      if (e != cudaSuccess) {
        c->graph_exec = nullptr;
        rc = int(e);
      }
    }
    if (g) cudaGraphDestroy(g);
    if (rc == 0) {
      e = cudaGraphLaunch(c->graph_exec, s);
      if (e != cudaSuccess) rc = int(e);
      c->last_graph = rc == 0;
    }
  }
  if (rc) return rc;
  c->graph_warm = true;
  return finish_rounds(c, P, s, learned, n_queries);
}

// A call's queries: the hexahedra's engine, then the primitive pass when the
// scene has prisms, quads or triangles. The primitive pass reads each
// query's hexahedron hit, so a call that asked for no hits gets a scratch
// array; a scene without hexahedra runs the primitive pass alone.
// The primitive pass, between two timing events when HO_OPT_TIME_ROUNDS is on.
static int timed_prims(ho_context* c, const TraceArgs& a, bool fresh, cudaStream_t s) {
  c->prim_timed = false;
  if (c->time_rounds) {
    for (cudaEvent_t& e : c->prim_events)
      if (!e && cudaEventCreate(&e) != cudaSuccess) return int(cudaGetLastError());
    const cudaError_t e = cudaEventRecord(c->prim_events[0], s);
    if (e != cudaSuccess) return int(e);
  }
  const int rc = launch_prims(c, a, a.hits, fresh, nullptr, s);
  if (rc || !c->time_rounds) return rc;
  const cudaError_t e = cudaEventRecord(c->prim_events[1], s);
  if (e != cudaSuccess) return int(e);
  c->prim_timed = true;
  return 0;
}

int launch_trace(ho_context* c, const TraceArgs& a_in, cudaStream_t s) {
  c->prim_timed = false;
  if (c->n_prims == 0) return trace_hexes(c, a_in, s);
  TraceArgs a = a_in;
  const int64_t nq = a.rays ? a.n_rays * a.n_iso
                            : (a.views ? a.n_queries_views : static_cast<int64_t>(a.width) * a.height * a.n_iso);
  if (nq == 0) return 0;
  if (!a.hits) {
    if (static_cast<size_t>(nq) > c->phits_cap || !c->d_phits) {
      cudaFree(c->d_phits);
      c->d_phits = nullptr;
      c->phits_cap = 0;
      const cudaError_t e = cudaMalloc(&c->d_phits, static_cast<size_t>(nq) * sizeof(ho_hit));
      if (e != cudaSuccess) return int(e);
      c->phits_cap = static_cast<size_t>(nq);
    }
    a.hits = c->d_phits;
  }
  if (c->n_elem == 0) {
    c->last_graph = false;
    c->stats_frozen = false;
    c->round_events_used = 0;
    c->launches = 1;
    return timed_prims(c, a, true, s);
  }
  const int rc = trace_hexes(c, a, s);
  if (rc) return rc;
  ++c->launches;
  return timed_prims(c, a, false, s);
}

}  // namespace ho
