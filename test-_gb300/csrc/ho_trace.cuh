// Ray queries against the curved-hex scene (plain mode).
//
// One thread per (ray, isovalue) query; for camera rays a warp covers an
// 8x4 pixel tile so the lanes of a warp mostly visit the same elements and
// their coefficient loads coalesce into broadcasts.
//
// Candidate order. The reference visits the elements whose padded box the
// ray meets in BVH stack order, clipping each candidate's segment to the
// closest hit found so far (FEM-AABB/raytracer.cu:111-358). Here candidates
// are visited in ascending (box entry t, element index) order with the same
// clipping: the traversal keeps the K smallest candidate keys above the last
// visited key in registers, visits them, and walks the tree again only when
// more than K candidates were in range (HO_FLAG_OVERFLOW), so every ray sees
// exactly the ordered candidate sequence whatever the tree shape.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include "ho_device.cuh"
#include "ho_fp64.cuh"
#include "ho_host.h"
#include "ho_learn.h"

namespace ho {

constexpr int kCandK = 8;
// learned mode: predictions for at most this many queued rays per call
constexpr int64_t kPredItemsCap = int64_t(8) << 20;
constexpr int kStack = 64;
constexpr int kTraceBlock = 128;  // intersect pass: 4 warps, one query each
constexpr int kGridCacheDevices = 64;  // devices whose persistent grid size launch_n caches



struct TraceParams {
  const BNode* __restrict__ nodes;
  const float* __restrict__ rec;
  const float* __restrict__ fbox;
  const float* __restrict__ box;
  const uint32_t* __restrict__ flags;
  const float* __restrict__ rays;  // explicit rays or nullptr
  int64_t n_rays;
  CamArgs cam;
  float iso[8];
  int n_iso;
  uint32_t iso_on_mask;
  const ViewDesc* views;  // multi-view call (rays == nullptr), else nullptr
  int n_views;
  ho_hit* __restrict__ hits;
  uint8_t* __restrict__ rgb;
  DevStats* stats;
  int32_t* work;      // queue of query indices that meet at least one box
  float2* kbuf;       // [queue slot][kCandK] first ordered candidates (t entry, element bits)
  uint8_t* kovf;      // [queue slot] more candidates than kCandK were in range
  unsigned* qcount;   // [0] queue length (classify pass), [2] rays with predictions
  unsigned pred_items;  // learned: predictions exist for queue items below this
  unsigned* qnext;    // next queue item to take (intersect pass)
  // learned mode
  const float* desc;      // element descriptors (scale k at [45])
  const int32_t* cand_e;  // [item][kPredK] candidate elements the predictions belong to
  const float* pred;      // [item][kPredK][8] network outputs
  int fp64;               // plain kernel: FP64 check + polish of every hit (HO_OPT_FP64_CHECK)
};

__device__ __forceinline__ bool key_less(float ta, int ea, float tb, int eb) {
  return ta < tb || (ta == tb && ea < eb);
}

// Insert (t, e) into the ascending register buffer; the largest falls out.
template <int K>
__device__ __forceinline__ void kbuf_insert(float (&bt)[K], int (&be)[K], float t, int e) {
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const bool sw = key_less(t, e, bt[j], be[j]);
    const float tt = sw ? bt[j] : t;
    const int ee = sw ? be[j] : e;
    bt[j] = sw ? t : bt[j];
    be[j] = sw ? e : be[j];
    t = tt;
    e = ee;
  }
}

__device__ __forceinline__ void load_child(const BNode* __restrict__ nodes, int node, int c, float (&lo)[3],
                                           float (&hi)[3], int& idx, uint32_t& aux) {
  const float4* p = reinterpret_cast<const float4*>(&nodes[node].c[c]);
  const float4 a = __ldg(p), b = __ldg(p + 1);
  lo[0] = a.x; lo[1] = a.y; lo[2] = a.z;
  idx = __float_as_int(a.w);
  hi[0] = b.x; hi[1] = b.y; hi[2] = b.z;
  aux = __float_as_uint(b.w);
}

// Collect the K smallest candidate keys > (kt, ke) with entry <= tmax from
// the tree `nodes`. Returns false on traversal-stack overflow (status set by
// the caller).
template <int K>
static __device__ bool collect_in(const BNode* __restrict__ nodes, float3 o, float3 d, float tmax, float kt, int ke,
                                  float (&bt)[K], int (&be)[K], bool& overflow, Work& w) {
#pragma unroll
  for (int j = 0; j < K; ++j) {
    bt[j] = FLT_MAX;
    be[j] = INT_MAX;
  }
  overflow = false;
  int stack[kStack];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const int node = stack[--sp];
    ++w.nodes;
    float te[2];
    int id[2];
    bool hit[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      float lo[3], hi[3];
      uint32_t aux;
      load_child(nodes, node, c, lo, hi, id[c], aux);
      hit[c] = false;
      te[c] = FLT_MAX;
      if (id[c] == kEmptyChild) continue;
      float a0, a1;
      if (!ray_box(o, d, lo, hi, 0.001f, tmax, a0, a1)) continue;
      if (a1 < kt) continue;  // everything inside enters before the last visited key
      // with the buffer full, a box entered after the K-th key holds only
      // candidates for a later walk: note that one is needed
      const bool full = be[K - 1] != INT_MAX;
      if (id[c] < 0) {
        const int e = ~id[c];
        if (!key_less(kt, ke, a0, e)) continue;  // already visited
        if (!key_less(a0, e, bt[K - 1], be[K - 1])) {
          overflow = true;
          continue;
        }
        if (full) overflow = true;  // the largest falls out
        kbuf_insert(bt, be, a0, e);
      } else if (full && a0 > bt[K - 1]) {
        overflow = true;
      } else {
        hit[c] = true;
        te[c] = a0;
      }
    }
    if (hit[0] && hit[1]) {
      if (sp + 2 > kStack) return false;
      const int nearc = te[0] <= te[1] ? 0 : 1;
      stack[sp++] = id[1 - nearc];
      stack[sp++] = id[nearc];
    } else if (hit[0] || hit[1]) {
      if (sp + 1 > kStack) return false;
      stack[sp++] = hit[0] ? id[0] : id[1];
    }
  }
  return true;
}

static __device__ __forceinline__ bool collect(const TraceParams& P, float3 o, float3 d, float tmax, float kt, int ke,
                                               float (&bt)[kCandK], int (&be)[kCandK], bool& overflow, Work& w) {
  return collect_in(P.nodes, o, d, tmax, kt, ke, bt, be, overflow, w);
}

__device__ __forceinline__ void flush_work(DevStats* st, const Work& w, bool active) {
  // warp-aggregated counters
  unsigned long long v[ST_FLUSH] = {active ? 1u : 0u, w.cand, w.geom, w.map, w.field, w.newton, w.face, w.culled,
                                    w.nodes, w.accepted, w.rejected, w.restarts, w.cyc[0], w.cyc[1], w.cyc[2],
                                    w.cyc[3], w.steps, w.lanes, 0ull, 0ull, 0ull, 0ull, 0ull, w.flops, 0ull};
#pragma unroll
  for (int s = 0; s < ST_FLUSH; ++s) {
    unsigned long long x = v[s];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(&st->c[s], x);
  }
}

// Primary-ray shading: Lambert headlight on hits (blue on face 0 as
// raytracer.cu:247-248 assigns material 1 there, grey otherwise), sky
// gradient on misses (raytracer.cu:398-402), gamma 2 and 8-bit quantisation
// (raytracer.cu:462-475).
__device__ __forceinline__ void shade(const HitState& h, float3 d, uint8_t* out) {
  float c[3];
  if (h.kind == HO_HIT_MISS) {
    const float a = 0.5f * (d.y + 1.0f);
    c[0] = (1.0f - a) * 1.0f + a * 0.5f;
    c[1] = (1.0f - a) * 1.0f + a * 0.7f;
    c[2] = (1.0f - a) * 1.0f + a * 1.0f;
  } else {
    const bool blue = h.kind == HO_HIT_FACE && h.face == 0;
    float lam = -(h.n.x * d.x + h.n.y * d.y + h.n.z * d.z);
    lam = lam > 0.f ? lam : 0.f;
    const float k = 0.2f + 0.8f * lam;
    c[0] = (blue ? 0.1f : 0.5f) * k;
    c[1] = (blue ? 0.2f : 0.5f) * k;
    c[2] = (blue ? 0.8f : 0.5f) * k;
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) out[q] = static_cast<uint8_t>(255.99f * fminf(1.0f, sqrtf(c[q])));
}

// Pixel-centre ray of pixel `pix` of a pinhole camera.
__device__ __forceinline__ void camera_ray(const CamArgs& cam, int64_t pix, float3& o, float3& d) {
  const int x = cam.x0 + static_cast<int>(pix % cam.width), y = cam.y0 + static_cast<int>(pix / cam.width);
  const float s = (static_cast<float>(x) + 0.5f) / static_cast<float>(cam.full_w);
  const float t = (static_cast<float>(y) + 0.5f) / static_cast<float>(cam.full_h);
  o = cam.origin;
  d = make_float3(cam.llc.x + s * cam.horiz.x + t * cam.vert.x - o.x, cam.llc.y + s * cam.horiz.y + t * cam.vert.y - o.y,
                  cam.llc.z + s * cam.horiz.z + t * cam.vert.z - o.z);
  d = normalize3(d);
}

// Rays as the kernels see them: query q -> (origin, direction, isovalue,
// isosurface on). Three layouts: explicit rays (isovalue-major over the ray
// array), one camera (isovalue-major over its pixels), or a table of views
// (each view's queries laid out like one camera, views back to back).
__device__ __forceinline__ void query_ray_from(const float* __restrict__ rays, int64_t n_rays, const CamArgs& cam,
                                               const float* iso_tab, uint32_t iso_mask, const ViewDesc* views,
                                               int n_views, int64_t q, float3& o, float3& d, float& iso,
                                               bool& iso_on) {
  int iso_idx;
  if (rays != nullptr) {
    iso_idx = static_cast<int>(q / n_rays);
    const float* rp = rays + 6 * (q - static_cast<int64_t>(iso_idx) * n_rays);
    o = make_float3(rp[0], rp[1], rp[2]);
    d = make_float3(rp[3], rp[4], rp[5]);
  } else if (views != nullptr) {
    int lo = 0, hi = n_views - 1;  // the last view whose first query <= q
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (views[mid].q0 <= q) lo = mid;
      else hi = mid - 1;
    }
    const ViewDesc& v = views[lo];
    const int64_t local = q - v.q0, npix = static_cast<int64_t>(v.cam.width) * v.cam.height;
    iso_idx = static_cast<int>(local / npix);
    camera_ray(v.cam, local - static_cast<int64_t>(iso_idx) * npix, o, d);
    iso = v.iso[iso_idx];
    iso_on = (v.iso_on_mask >> iso_idx) & 1u;
    return;
  } else {
    const int64_t npix = static_cast<int64_t>(cam.width) * cam.height;
    iso_idx = static_cast<int>(q / npix);
    camera_ray(cam, q - static_cast<int64_t>(iso_idx) * npix, o, d);
  }
  iso = iso_tab[iso_idx];
  iso_on = (iso_mask >> iso_idx) & 1u;
}

__device__ __forceinline__ void query_ray(const TraceParams& P, int64_t q, float3& o, float3& d, float& iso,
                                          bool& iso_on) {
  query_ray_from(P.rays, P.n_rays, P.cam, P.iso, P.iso_on_mask, P.views, P.n_views, q, o, d, iso, iso_on);
}

// A hit whose ray meets the surface at |cos| below this is grazing: there a
// rounding can move the hit to a neighbouring face or element, or off the
// surface (HO_FLAG_GRAZING, ho_stats.grazing_hits).
constexpr float kGrazeCos = 0.05f;
__device__ __forceinline__ bool is_grazing(const HitState& b, float3 d) {
  if (b.kind == HO_HIT_MISS) return false;
  const float dn = fabsf(b.n.x * d.x + b.n.y * d.y + b.n.z * d.z);
  return dn < kGrazeCos * sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
}

__device__ __forceinline__ void write_result(const TraceParams& P, int64_t q, float3 d, const HitState& best,
                                             uint32_t iters) {
  if (P.hits) {
    ho_hit h;
    h.t = best.t;
    h.elem = best.elem;
    h.face = static_cast<int16_t>(best.face);
    h.kind = static_cast<int16_t>(best.kind);
    h.xi[0] = best.xi.x; h.xi[1] = best.xi.y; h.xi[2] = best.xi.z;
    h.n[0] = best.n.x; h.n[1] = best.n.y; h.n[2] = best.n.z;
    h.u = best.u;
    h.flags = best.flags | (is_grazing(best, d) ? HO_FLAG_GRAZING : 0u);
    h.iters = iters;
    P.hits[q] = h;
  }
  if (P.rgb && P.rays == nullptr) shade(best, d, P.rgb + 3 * q);
}

__device__ __forceinline__ HitState miss_state() {
  HitState b;
  b.t = FLT_MAX;
  b.elem = -1;
  b.face = -1;
  b.kind = HO_HIT_MISS;
  b.xi = make_float3(0.f, 0.f, 0.f);
  b.n = b.xi;
  b.u = 0.f;
  b.flags = 0;
  return b;
}

// Pass 2, persistent, one warp per queued query: ordered candidates, each
// visited with its independent Newton solves spread over the lanes.
template <int N, bool LEARNED>
__global__ void __launch_bounds__(kTraceBlock) isect_kernel(TraceParams P) {
  const int lane = threadIdx.x & 31;
  // one staging slot per warp for the element record being visited
  extern __shared__ __align__(16) float stage[];
  float4* slot4 = reinterpret_cast<float4*>(stage + (threadIdx.x >> 5) * record_floats(N));
  const uint32_t slot_addr = static_cast<uint32_t>(__cvta_generic_to_shared(slot4));
  Work w, wu;
  const unsigned n_work = *P.qcount;
  for (;;) {
    unsigned item = 0;
    if (lane == 0) item = atomicAdd(P.qnext, 1u);
    item = __shfl_sync(kFull, item, 0);
    if (item >= n_work) break;
    const int64_t q = P.work[item];
    float3 o, d;
    float iso;
    bool iso_on;
    query_ray(P, q, o, d, iso, iso_on);
    HitState best = miss_state();
    const uint32_t it0 = wu.newton + wu.face + w.newton + w.face;
    float kt = -FLT_MAX;
    int ke = -1;
    int pass = 0;
    for (;;) {
      float bt[kCandK];
      int be[kCandK];
      bool overflow;
      const long long c0 = clock64();
      bool walked = true;
      if (pass == 0) {
        // the classify pass already walked the tree for this ray
        const float2* kb = P.kbuf + static_cast<int64_t>(item) * kCandK;
#pragma unroll
        for (int j = 0; j < kCandK; ++j) {
          const float2 c = kb[j];
          bt[j] = c.x;
          be[j] = __float_as_int(c.y);
        }
        overflow = P.kovf[item] != 0;
      } else {
        walked = collect(P, o, d, best.t, kt, ke, bt, be, overflow, wu);
      }
      wu.cyc[0] += clock64() - c0;
      if (!walked) {
        if (lane == 0) atomicOr(&P.stats->status, kStatusStackOverflow);
        best.flags |= HO_FLAG_INCOMPLETE;
        break;
      }
      bool done = false;
#pragma unroll 1
      for (int j = 0; j < kCandK; ++j) {
        float ct = bt[0];
        int ce = be[0];
#pragma unroll
        for (int m = 1; m < kCandK; ++m)
          if (j == m) {
            ct = bt[m];
            ce = be[m];
          }
        if (ce == INT_MAX || ct > best.t) {
          done = true;
          break;
        }
        const float* b = P.box + 6 * static_cast<int64_t>(ce);
        const float lo[3] = {__ldg(b), __ldg(b + 1), __ldg(b + 2)};
        const float hi[3] = {__ldg(b + 3), __ldg(b + 4), __ldg(b + 5)};
        float te, tx;
        if (ray_box(o, d, lo, hi, 0.001f, best.t, te, tx)) {
          // stage the candidate's record in this warp's shared-memory slot
          const float4* src = reinterpret_cast<const float4*>(P.rec + static_cast<int64_t>(ce) * record_floats(N));
          __syncwarp();
          for (int q4 = lane; q4 < record_floats(N) / 4; q4 += 32) slot4[q4] = __ldg(src + q4);
          __syncwarp();
          Elem<N, true> el;
          el.c = CoefRef<true>{slot_addr};
          el.has_field = (__ldg(P.flags + ce) & 1u) != 0;
          Pred pr;
          pr.on = false;
          if (LEARNED && pass == 0 && j < kPredK && P.cand_e[static_cast<int64_t>(item) * kPredK + j] == ce) {
            const float* y = P.pred + (static_cast<int64_t>(item) * kPredK + j) * kMlpOut;
            pr.on = true;
            pr.xi_in = make_float3(y[0], y[1], y[2]);
            pr.v = make_float3(y[3], y[4], y[5]);
            pr.k = __ldg(P.desc + static_cast<int64_t>(ce) * kDescFloats + 45);
            pr.te = te;
          }
          visit_warp<N, LEARNED>(el, P.fbox + static_cast<int64_t>(ce) * kFaceBoxFloats, ce, o, d, te, tx, iso,
                                 iso_on, best, w, wu, pr);
        }
        kt = ct;
        ke = ce;
      }
      if (done || !overflow) break;
      ++wu.restarts;
      ++pass;
      best.flags |= HO_FLAG_OVERFLOW;
    }
    // iterations of this query summed over the lanes
    uint32_t its = w.newton + w.face;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) its += __shfl_xor_sync(kFull, its, off);
    if (lane == 0) write_result(P, q, d, best, its + wu.newton + wu.face - it0);
  }
  if (lane == 0) {
    w.cand += wu.cand; w.geom += wu.geom; w.map += wu.map; w.field += wu.field; w.newton += wu.newton;
    w.face += wu.face; w.culled += wu.culled; w.nodes += wu.nodes; w.restarts += wu.restarts;
    w.accepted += wu.accepted; w.rejected += wu.rejected;
    for (int k = 0; k < 4; ++k) w.cyc[k] = wu.cyc[k];
  }
  flush_work(P.stats, w, false);
}

// The reference's per-ray structure: ordered candidates, each visited with
// the sequential cold-start algorithm (visit_candidate), walking the tree
// again when more than kCandK candidates were in range.
template <int N>
__device__ HitState plain_trace(const TraceParams& P, float3 o, float3 d, float iso, bool iso_on, Work& w,
                                HitState* tie = nullptr) {
  HitState best = miss_state();
  if (tie) *tie = miss_state();
  float kt = -FLT_MAX;
  int ke = -1;
  for (;;) {
    float bt[kCandK];
    int be[kCandK];
    bool overflow;
    if (!collect(P, o, d, best.t, kt, ke, bt, be, overflow, w)) {
      atomicOr(&P.stats->status, kStatusStackOverflow);
      best.flags |= HO_FLAG_INCOMPLETE;
      break;
    }
    bool done = false;
#pragma unroll 1
    for (int j = 0; j < kCandK; ++j) {
      float ct = bt[0];
      int ce = be[0];
#pragma unroll
      for (int m = 1; m < kCandK; ++m)
        if (j == m) {
          ct = bt[m];
          ce = be[m];
        }
      if (ce == INT_MAX || ct > best.t) {
        done = true;
        break;
      }
      const float* b = P.box + 6 * static_cast<int64_t>(ce);
      const float lo[3] = {__ldg(b), __ldg(b + 1), __ldg(b + 2)};
      const float hi[3] = {__ldg(b + 3), __ldg(b + 4), __ldg(b + 5)};
      float te, tx;
      if (ray_box(o, d, lo, hi, 0.001f, best.t, te, tx)) {
        Elem<N> el;
        el.c = CoefRef<false>{P.rec + static_cast<int64_t>(ce) * record_floats(N)};
        el.has_field = (__ldg(P.flags + ce) & 1u) != 0;
        visit_candidate<N>(el, P.fbox + static_cast<int64_t>(ce) * kFaceBoxFloats, ce, o, d, te, tx, iso, iso_on, best,
                           w, tie);
      }
      kt = ct;
      ke = ce;
    }
    if (done || !overflow) break;
    ++w.restarts;
    best.flags |= HO_FLAG_OVERFLOW;
  }
  return best;
}

// Plain form: the reference's structure on the GPU — one thread per query
// (camera rays: a warp covers an 8x4 pixel tile), no queue, no lane-parallel
// solves, no prediction.
template <int N>
__global__ void __launch_bounds__(kTraceBlock) plain_kernel(TraceParams P, int64_t n_queries) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = (static_cast<int64_t>(blockIdx.x) * kTraceBlock + threadIdx.x) >> 5;
  int64_t q;
  float3 o = make_float3(0.f, 0.f, 0.f), d = make_float3(0.f, 0.f, 1.f);
  float iso = 0.f;
  bool iso_on = false;
  bool active;
  if (P.rays == nullptr && P.views == nullptr) {
    const int tx_n = (P.cam.width + 7) >> 3, ty_n = (P.cam.height + 3) >> 2;
    const int64_t tiles = static_cast<int64_t>(tx_n) * ty_n;
    const int it = static_cast<int>(wid / tiles);
    const int64_t tile = wid - static_cast<int64_t>(it) * tiles;
    const int x = static_cast<int>(tile % tx_n) * 8 + (lane & 7);
    const int y = static_cast<int>(tile / tx_n) * 4 + (lane >> 3);
    active = it < P.n_iso && x < P.cam.width && y < P.cam.height;
    q = static_cast<int64_t>(it) * P.cam.width * P.cam.height + static_cast<int64_t>(y) * P.cam.width + x;
  } else {
    q = static_cast<int64_t>(blockIdx.x) * kTraceBlock + threadIdx.x;
    active = q < n_queries;
  }
  if (active) query_ray(P, q, o, d, iso, iso_on);
  Work w;
  HitState best = miss_state();
  bool polished = false;
  int tie_seen = 0, tie_swapped = 0;
  if (active) {
    HitState tie;
    best = plain_trace<N>(P, o, d, iso, iso_on, w, &tie);
    // the FP64 check, polish and tie rule of the engines' final pass; the
    // plain solver is the fallback itself, so a failing hit is only flagged
    if (P.fp64) {
      double t64;
      if (!fp64_check_polish<N>(P.rec, P.flags, o, d, iso, best, polished, &t64)) {
        best.flags |= HO_FLAG_FP64_FAIL;
      } else if (tie.kind != HO_HIT_MISS) {
        tie_seen = 1;
        tie_swapped = fp64_tie_rule<N>(P.rec, P.flags, o, d, iso, best, t64, tie) ? 1 : 0;
      }
    }
  }
  flush_work(P.stats, w, active);
  const unsigned pm = __ballot_sync(kFull, polished), tm = __ballot_sync(kFull, tie_seen),
                 sm = __ballot_sync(kFull, tie_swapped), gm = __ballot_sync(kFull, active && is_grazing(best, d));
  if ((threadIdx.x & 31) == 0) {
    if (gm) atomicAdd(&P.stats->c[ST_GRAZING], static_cast<unsigned long long>(__popc(gm)));
    if (pm) atomicAdd(&P.stats->c[ST_POLISHED], static_cast<unsigned long long>(__popc(pm)));
    if (tm) atomicAdd(&P.stats->c[ST_TIES], static_cast<unsigned long long>(__popc(tm)));
    if (sm) atomicAdd(&P.stats->c[ST_TIES_SWAPPED], static_cast<unsigned long long>(__popc(sm)));
  }
  if (active) write_result(P, q, d, best, w.newton + w.face);
}

template <int N>
cudaError_t launch_n(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode) {
  if (mode == HO_MODE_PLAIN) {
    const int64_t blocks = (n_threads + kTraceBlock - 1) / kTraceBlock;
    plain_kernel<N><<<static_cast<unsigned>(blocks), kTraceBlock, 0, s>>>(P, n_queries);
    return cudaGetLastError();
  }
  const bool learned = mode == HO_MODE_LEARNED;
  // persistent grid (resident blocks per SM x SMs), per device and form; two
  // host threads that fill the same entry at once store the same value
  static std::atomic<int> grid[kGridCacheDevices][2];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kGridCacheDevices) return cudaErrorInvalidDevice;
  int g = grid[dev][learned ? 1 : 0].load(std::memory_order_acquire);
  if (g == 0) {
    const int smem_i = static_cast<int>((kTraceBlock / 32) * record_floats(N) * sizeof(float));
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (learned) {
      cudaFuncSetAttribute(isect_kernel<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_i);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, isect_kernel<N, true>, kTraceBlock, smem_i);
    } else {
      cudaFuncSetAttribute(isect_kernel<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_i);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, isect_kernel<N, false>, kTraceBlock, smem_i);
    }
    g = sms * (per > 0 ? per : 1);
    grid[dev][learned ? 1 : 0].store(g, std::memory_order_release);
  }
  const size_t smem = static_cast<size_t>(kTraceBlock / 32) * record_floats(N) * sizeof(float);
  if (learned) isect_kernel<N, true><<<g, kTraceBlock, smem, s>>>(P);
  else isect_kernel<N, false><<<g, kTraceBlock, smem, s>>>(P);
  return cudaGetLastError();
}

// explicit instantiations live in ho_trace_n*.cu
extern template cudaError_t launch_n<2>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
extern template cudaError_t launch_n<3>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
extern template cudaError_t launch_n<4>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
extern template cudaError_t launch_n<5>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
extern template cudaError_t launch_n<6>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
extern template cudaError_t launch_n<7>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
extern template cudaError_t launch_n<8>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);
extern template cudaError_t launch_n<9>(const TraceParams& P, int64_t n_queries, int64_t n_threads, cudaStream_t s, int mode);

}  // namespace ho
