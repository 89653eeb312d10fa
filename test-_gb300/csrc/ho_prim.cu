// Prisms, quads and curved triangles: upload, sampled boxes, their own
// LBVH, and the primitive pass of a trace call.
//
// The reference traces every primitive kind in one BVH walk
// (FEM-AABB/raytracer.cu:255-347). Here the hexahedra go through their own
// engine first; the primitive pass then visits, per query, the primitives
// whose box the ray meets in ascending (box entry, index) order, each on the
// segment [0.001, closest hit so far] that starts at the hexahedra's hit,
// and keeps a primitive hit when it is nearer. One thread per query: the
// per-primitive solves are short, branchy FP32 Newton loops whose start
// search the reference defines by exact comparisons. This file is compiled
// without multiply-add contraction (see ho_prim.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "ho_host.h"
#include "ho_prim.cuh"
#include "ho_trace.cuh"

namespace ho {

namespace {

#define PR_TRY(x)                            \
  do {                                       \
    cudaError_t e__ = (x);                   \
    if (e__ != cudaSuccess) return int(e__); \
  } while (0)

constexpr int kPrimThreads = 128;
// Resident blocks per SM the register budget is sized for (80 registers a
// thread; measured faster than 64, 128 or an unbounded 208 despite spills),
// and candidates collected per walk of the primitive tree (a ray with more
// walks again; 16 halves the node visits but measured no faster).
#ifndef HO_PRIM_MIN_BLOCKS
#define HO_PRIM_MIN_BLOCKS 6
#endif
#ifndef HO_PRIM_CAND_K
#define HO_PRIM_CAND_K 8
#endif
constexpr int kPrimCandK = HO_PRIM_CAND_K;

__global__ void prim_setup_kernel(PrimRec* __restrict__ recs, const float* __restrict__ pool, int64_t n,
                                  float* __restrict__ box) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PrimRec p = recs[i];
  float lo[3], hi[3];
  pr_box(p, pool, lo, hi);
  for (int a = 0; a < 3; ++a) {
    recs[i].lo[a] = lo[a];
    recs[i].hi[a] = hi[a];
    box[6 * i + a] = lo[a];
    box[6 * i + 3 + a] = hi[a];
  }
}

struct PrimParams {
  const BNode* __restrict__ nodes;
  const PrimRec* __restrict__ prims;
  const float* __restrict__ geom;
  const float* __restrict__ field;
  const float* __restrict__ rays;
  int64_t n_rays;
  CamArgs cam;
  const ViewDesc* views;
  int n_views;
  float iso[8];
  uint32_t iso_mask;
  ho_hit* __restrict__ hits;
  uint8_t* __restrict__ rgb;
  int64_t n_queries;
  bool fresh;
  DevStats* stats;
};

// One query's primitive pass: the candidates in (box entry, index) order on
// [0.001, closest hit so far], then the hit record and the pixel.
__device__ __forceinline__ void prim_query(const PrimParams& P, int64_t q, PrimWork& pw, unsigned& cand, Work& w) {
  float3 o, d;
  float iso;
  bool iso_on;
  query_ray_from(P.rays, P.n_rays, P.cam, P.iso, P.iso_mask, P.views, P.n_views, q, o, d, iso, iso_on);
  ho_hit h;
  if (P.fresh) {
    h.t = FLT_MAX;
    h.elem = -1;
    h.face = -1;
    h.kind = HO_HIT_MISS;
    for (int a = 0; a < 3; ++a) h.xi[a] = h.n[a] = 0.f;
    h.u = 0.f;
    h.flags = 0;
    h.iters = 0;
  } else {
    h = P.hits[q];
  }
  float best = h.kind != HO_HIT_MISS ? h.t : FLT_MAX;
  int win = -1;
  float3 xw = make_float3(0.f, 0.f, 0.f);
  const uint32_t iters0 = pw.iters;
  float kt = -FLT_MAX;
  int ke = -1;
  bool incomplete = false;
  for (;;) {
    float bt[kPrimCandK];
    int be[kPrimCandK];
    bool overflow;
    if (!collect_in<kPrimCandK>(P.nodes, o, d, best, kt, ke, bt, be, overflow, w)) {
      atomicOr(&P.stats->status, kStatusStackOverflow);
      incomplete = true;
      break;
    }
    bool done = false;
#pragma unroll 1
    for (int j = 0; j < kPrimCandK; ++j) {
      float ct = bt[0];
      int ce = be[0];
#pragma unroll
      for (int m = 1; m < kPrimCandK; ++m)
        if (j == m) {
          ct = bt[m];
          ce = be[m];
        }
      if (ce == INT_MAX || ct > best) {
        done = true;
        break;
      }
      const PrimRec& p = P.prims[ce];  // read in place: the solvers take it by reference
      float te, tx, th;
      float3 xh;
      ++cand;
      if (pr_slab(o, d, p.lo, p.hi, 0.001f, best, te, tx) && pr_hit(p, P.geom, o, d, 0.001f, best, th, xh, pw) &&
          th > 0.001f && th < best) {
        best = th;
        win = ce;
        xw = xh;
      }
      kt = ct;
      ke = ce;
    }
    if (done || !overflow) break;
  }
  if (win >= 0) {
    const PrimRec& p = P.prims[win];
    const float3 n = pr_normal(p, P.geom, xw, d);
    h.t = best;
    h.elem = p.local;
    h.face = -1;
    h.kind = static_cast<int16_t>(HO_HIT_PRISM + p.kind);
    h.xi[0] = xw.x;
    h.xi[1] = xw.y;
    h.xi[2] = xw.z;
    h.n[0] = n.x;
    h.n[1] = n.y;
    h.n[2] = n.z;
    h.u = pr_field(p, P.field, xw);
    h.flags = 0;
  }
  h.iters += pw.iters - iters0;
  if (incomplete) h.flags |= HO_FLAG_INCOMPLETE;
  if (P.hits && (P.fresh || win >= 0 || incomplete)) P.hits[q] = h;
  if (P.rgb && P.rays == nullptr && (P.fresh || win >= 0)) {
    HitState s;
    s.t = h.t;
    s.elem = h.elem;
    s.face = h.face;
    s.kind = h.kind;
    s.n = make_float3(h.n[0], h.n[1], h.n[2]);
    shade(s, d, P.rgb + 3 * q);
  }
}

__global__ void __launch_bounds__(kPrimThreads, HO_PRIM_MIN_BLOCKS) prim_trace_kernel(PrimParams P) {
  PrimWork pw;
  unsigned cand = 0;
  Work w;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q < P.n_queries) prim_query(P, q, pw, cand, w);
  // counters: summed over the warp when all its lanes are here together
  // (the last block's tail warp is partial), else added one by one
  const unsigned long long v[4] = {cand, pw.iters, pw.flops, w.nodes};
  const bool whole = __activemask() == 0xffffffffu;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    unsigned long long x = v[k];
    if (whole) {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
      if ((threadIdx.x & 31) != 0) x = 0;
    }
    if (x) atomicAdd(&P.stats->c[ST_PRIM_CAND + k], x);
  }
}

// Host copy of the primitives, kind-major, with modes packed and offsets
// rebased; a geometry whose modes do not make it curved for its kind is
// kept linear, as the reference's HasHighOrderGeom decides.
void pack_prims(const HostPrims& hp, std::vector<PrimRec>& recs, int64_t counts[3]) {
  recs.clear();
  counts[0] = counts[1] = counts[2] = 0;
  for (int k = 0; k < 3; ++k)
    for (int64_t i = 0; i < hp.size(); ++i) {
      if (hp.kind[i] != k) continue;
      PrimRec r;
      std::memset(&r, 0, sizeof(r));
      std::copy(hp.verts.begin() + 18 * i, hp.verts.begin() + 18 * i + 18, r.v);
      r.kind = k;
      r.local = static_cast<int32_t>(counts[k]++);
      const uint32_t* g = hp.gmodes.data() + 3 * i;
      const uint32_t* f = hp.fmodes.data() + 3 * i;
      const bool curved = hp.goff[i] >= 0 && g[0] > 0 && g[1] > 0 && (k != kPrimPrism || g[2] > 0);
      r.gm = curved ? (g[0] | g[1] << 8 | (k == kPrimPrism ? g[2] : 0u) << 16) : 0u;
      r.goff = curved ? hp.goff[i] : -1;
      r.fm = f[0] | f[1] << 8 | (k == kPrimPrism ? f[2] : 0u) << 16;
      r.foff = hp.foff[i];
      recs.push_back(r);
    }
}

}  // namespace

void prims_free(ho_context* c) {
  cudaFree(c->d_prims);
  cudaFree(c->d_pgeom);
  cudaFree(c->d_pfield);
  cudaFree(c->d_pbox);
  cudaFree(c->d_pnodes);
  c->d_prims = nullptr;
  c->d_pgeom = c->d_pfield = c->d_pbox = nullptr;
  c->d_pnodes = nullptr;
  c->n_prims = c->n_pnodes = 0;
  c->pbvh_depth = 0;
  c->prim_counts[0] = c->prim_counts[1] = c->prim_counts[2] = 0;
}

int prims_build(ho_context* c) {
  prims_free(c);
  const HostPrims& hp = c->hs.prims;
  if (hp.size() == 0) return 0;
  std::vector<PrimRec> recs;
  pack_prims(hp, recs, c->prim_counts);
  const int64_t n = static_cast<int64_t>(recs.size());
  cudaStream_t s = c->stream;
  const size_t ng = std::max<size_t>(hp.geom.size(), 1), nf = std::max<size_t>(hp.field.size(), 1);
  PR_TRY(cudaMalloc(&c->d_prims, n * sizeof(PrimRec)));
  PR_TRY(cudaMalloc(&c->d_pgeom, ng * sizeof(float)));
  PR_TRY(cudaMalloc(&c->d_pfield, nf * sizeof(float)));
  PR_TRY(cudaMalloc(&c->d_pbox, n * 6 * sizeof(float)));
  PR_TRY(cudaMemcpyAsync(c->d_prims, recs.data(), n * sizeof(PrimRec), cudaMemcpyHostToDevice, s));
  if (!hp.geom.empty())
    PR_TRY(cudaMemcpyAsync(c->d_pgeom, hp.geom.data(), hp.geom.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  if (!hp.field.empty())
    PR_TRY(cudaMemcpyAsync(c->d_pfield, hp.field.data(), hp.field.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  prim_setup_kernel<<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(static_cast<PrimRec*>(c->d_prims),
                                                                           c->d_pgeom, n, c->d_pbox);
  PR_TRY(cudaGetLastError());
  float bounds[6];
  const int rc = build_tree(c->d_pbox, nullptr, n, s, &c->d_pnodes, &c->n_pnodes, &c->pbvh_depth, bounds);
  if (rc) return rc;
  c->n_prims = n;
  c->device_bytes += n * static_cast<int64_t>(sizeof(PrimRec) + 24 + sizeof(BNode)) +
                     static_cast<int64_t>((ng + nf) * sizeof(float));
  return 0;
}

int launch_prims(ho_context* c, const TraceArgs& a, ho_hit* hits, bool fresh, DevStats* stats, cudaStream_t s) {
  PrimParams P;
  P.nodes = c->d_pnodes;
  P.prims = static_cast<const PrimRec*>(c->d_prims);
  P.geom = c->d_pgeom;
  P.field = c->d_pfield;
  P.rays = a.rays;
  P.n_rays = a.n_rays;
  P.cam = cam_args(a);
  P.views = a.views;
  P.n_views = a.n_views;
  for (int i = 0; i < 8; ++i) P.iso[i] = i < a.n_iso ? a.iso[i] : 0.f;
  P.iso_mask = a.iso_on_mask;
  P.hits = hits;
  P.rgb = a.rgb;
  P.n_queries = a.rays ? a.n_rays * a.n_iso
                       : (a.views ? a.n_queries_views : static_cast<int64_t>(a.width) * a.height * a.n_iso);
  P.fresh = fresh;
  P.stats = stats ? stats : c->d_stats;
  if (P.n_queries == 0) return 0;
  const int64_t blocks = (P.n_queries + kPrimThreads - 1) / kPrimThreads;
  prim_trace_kernel<<<static_cast<unsigned>(blocks), kPrimThreads, 0, s>>>(P);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace ho
