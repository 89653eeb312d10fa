// Dispatch of the trace kernel by modes per direction; each instantiation
// lives in its own translation unit (ho_trace_n*.cu) so they compile in
// parallel.
#include <algorithm>

#include "ho_trace.cuh"

namespace ho {

// Pass 1, one thread per query: rays that meet no padded box are finished
// here (miss); the rest are appended to the work queue together with their
// first kCandK ordered candidates.
__global__ void __launch_bounds__(256) classify_kernel(TraceParams P, int64_t n_queries) {
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  Work w;
  bool need = false, overflow = false;
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
    }
    need = be[0] != INT_MAX;
    if (!need) write_result(P, q, d, miss_state(), 0);
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

// Learned mode, after classify: the first kPredK ordered candidates of each
// queued ray (the same as the intersect pass's first candidates: nothing is
// hit yet) and the network input of each (ray, candidate) pair.
__global__ void __launch_bounds__(128) cand_kernel(TraceParams P, __nv_bfloat16* __restrict__ X,
                                                   int32_t* __restrict__ cand_e) {
  // predictions for the first pred_items queued rays (the buffers' size); the
  // rest start cold
  const unsigned n_work = min(*P.qcount, P.pred_items);
  if (blockIdx.x == 0 && threadIdx.x == 0) P.qcount[2] = n_work;
  Work w;
  for (int64_t item = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; item < n_work;
       item += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t q = P.work[item];
    float3 o, d;
    float iso;
    bool iso_on;
    query_ray(P, q, o, d, iso, iso_on);
    const float2* kb = P.kbuf + item * kCandK;
#pragma unroll
    for (int j = 0; j < kPredK; ++j) {
      const float2 c = kb[j];
      const int ce = __float_as_int(c.y);
      const int e = ce != INT_MAX ? ce : -1;
      cand_e[item * kPredK + j] = e;
      __nv_bfloat16* row = X + (item * kPredK + j) * kMlpInPad;
      if (e >= 0) {
        write_features(P.desc + static_cast<int64_t>(e) * kDescFloats, o, d, c.x, row);
      } else {
        for (int c = 0; c < kMlpInPad; ++c) row[c] = __float2bfloat16(0.f);
      }
    }
  }
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
    c->launches += 2;
    cand_kernel<<<sms * 8, 128, 0, s>>>(P, static_cast<__nv_bfloat16*>(c->d_feat), c->d_cand);
    e = cudaGetLastError();
    if (e != cudaSuccess) return int(e);
    const int rc = mlp_infer(c->mlp.dev(), c->d_feat, 0, c->d_qctr + 2, kPredK, c->d_pred, s, sms);
    if (rc) return rc;
  }
  // as many rounds as the previous call needed, plus one, within the option
  const int rounds = c->rounds_needed > 0 ? std::min(c->round_count, c->rounds_needed + 1) : c->round_count;
  return enqueue_rounds(c, P, s, learned, n_queries, rounds);
}

int launch_trace(ho_context* c, const TraceArgs& a, cudaStream_t s) {
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
  P.cam.origin = make_float3(a.origin[0], a.origin[1], a.origin[2]);
  P.cam.llc = make_float3(a.llc[0], a.llc[1], a.llc[2]);
  P.cam.horiz = make_float3(a.horiz[0], a.horiz[1], a.horiz[2]);
  P.cam.vert = make_float3(a.vert[0], a.vert[1], a.vert[2]);
  P.cam.width = a.width;
  P.cam.height = a.height;
  for (int i = 0; i < 8; ++i) P.iso[i] = i < a.n_iso ? a.iso[i] : 0.f;
  P.n_iso = a.n_iso;
  P.iso_on_mask = a.iso_on_mask;
  P.views = a.views;
  P.n_views = a.n_views;
  P.hits = a.hits;
  P.rgb = a.rgb;
  P.stats = c->d_stats;
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
      cudaFree(c->d_feat);
      cudaFree(c->d_pred);
      cudaFree(c->d_cand);
      c->d_feat = nullptr;
      c->d_pred = nullptr;
      c->d_cand = nullptr;
      c->pred_cap = 0;
      cudaError_t e = cudaMalloc(&c->d_feat, rows * kMlpInPad * sizeof(__nv_bfloat16));
      if (e == cudaSuccess) e = cudaMalloc(&c->d_pred, rows * kMlpOut * sizeof(float));
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

}  // namespace ho
