// Dispatch of the trace kernel by modes per direction; each instantiation
// lives in its own translation unit (ho_trace_n*.cu) so they compile in
// parallel.
#include "ho_trace.cuh"

namespace ho {

int launch_trace(ho_context* c, const TraceArgs& a, cudaStream_t s) {
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
  P.hits = a.hits;
  P.rgb = a.rgb;
  P.stats = c->d_stats;
  int64_t n_queries, n_threads;
  if (a.rays) {
    n_queries = a.n_rays * a.n_iso;
    n_threads = n_queries;
  } else {
    const int64_t tiles = static_cast<int64_t>((a.width + 7) / 8) * ((a.height + 3) / 4);
    n_queries = static_cast<int64_t>(a.width) * a.height * a.n_iso;
    n_threads = tiles * 32 * a.n_iso;
  }
  if (n_threads == 0) return 0;
  cudaError_t e;
  switch (c->N) {
    case 2: e = launch_n<2>(P, n_queries, n_threads, s); break;
    case 3: e = launch_n<3>(P, n_queries, n_threads, s); break;
    case 4: e = launch_n<4>(P, n_queries, n_threads, s); break;
    case 5: e = launch_n<5>(P, n_queries, n_threads, s); break;
    case 6: e = launch_n<6>(P, n_queries, n_threads, s); break;
    case 7: e = launch_n<7>(P, n_queries, n_threads, s); break;
    case 8: e = launch_n<8>(P, n_queries, n_threads, s); break;
    case 9: e = launch_n<9>(P, n_queries, n_threads, s); break;
    default: return int(cudaErrorInvalidValue);
  }
  return int(e);
}

}  // namespace ho
