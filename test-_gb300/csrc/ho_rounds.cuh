// Element-major intersection rounds (batched and learned modes).
//
// The per-candidate algorithm is the reference's hex branch
// (FEM-AABB/raytracer.cu:184-254): isosurface scan of 17 samples on the
// candidate's padded-box segment with bracket refinement
// (FEM-AABB/fem/RayIsosurface.cu:67-188); when that finds no root, the
// nearest curved-face hit over the 6 faces from 9 seeds each
// (FEM-AABB/high_order.h:189-304, 409-465). Every step is a Newton solve
// whose iterations each evaluate the element's geometry (x and J).
//
// How the work is laid out here. A round takes, for every ray still in
// flight, its next ordered candidate (ascending box entry, element index),
// so a round's (ray, element) pairs are independent. The pairs are bucketed
// by element, and one warp takes a batch of up to B pairs of one element:
// the element's record is staged in the warp's shared memory once, and the
// Newton solves of all its pairs (17 samples each, the refinement, the
// learned face start, the face seeds) are tasks in a warp-local queue. Each
// lane runs one solve at a time; every loop iteration all busy lanes
// evaluate the geometry at their own point (the same code, so the warp stays
// converged), then advance their own solve; a lane whose solve ends takes
// the next task. Tasks that depend on others (a pair's refinement or face
// search after its 17 samples) are queued by the lane that finishes the
// last task they depend on.
//
// With cold starts (batched mode) the results equal the warp-per-ray
// kernel's: the same solves with the same start points, iteration caps and
// acceptance rules, the same bracket (first sign change in sample order) and
// the same face choice (per face the lowest accepted seed index, faces
// compared in index order). With network starts (learned mode) a failed warm
// start restarts from whichever neighbouring sample has converged by then,
// so the two kernels agree to the solvers' tolerance.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "ho_device.cuh"
#include "ho_host.h"
#include "ho_learn.h"
#include "ho_tc.cuh"
#include "ho_trace.cuh"

namespace ho {

constexpr int kRoundBlock = 128;  // 4 warps, one batch each
constexpr int kSamples = 17;

// Pairs per batch (HO_OPT_ROUND_CHUNK, default the slot count): a warp admits
// a batch's pairs into its slots as earlier pairs finish, so a batch may be
// several times the slot count; smaller batches spread an element's pairs
// over more warps, which evens out the end of a round.

template <int N>
struct RoundCfg {
  static constexpr int B = round_slots(N);  // pair slots
  static constexpr int Ring = B * 56;         // task queue entries (>= B*54 face seeds)
};

// A (ray, candidate) pair of one round, as the gather pass writes it.
struct RoundPair {
  int32_t item;  // queue item (ray)
  int32_t j;     // index of the candidate in the ray's list (learned prediction lookup)
  float te, tx;  // segment: the candidate's padded box clipped to [0.001, closest hit]
};

struct RoundBatch {
  int32_t elem;
  int32_t first;  // into the element-sorted pairs
  int32_t count;
  int32_t pad;
};

// Per queue item state kept across rounds.
struct RayState {
  HitState best;
  HitState tie;  // the hit the best one displaced within kTieT (else a miss)
  int cursor;   // next candidate in the item's list
  int pass;     // 0: the classify pass's list (with predictions); >0 re-collected
  float kt;     // last visited key (entry t, element)
  int ke;
  int done;
  int ovf;      // the current list was cut at kCandK candidates
  int its;      // Newton and face iterations spent on the ray
  int pad;
};

struct RoundParams {
  const float* __restrict__ rec;
  const float* __restrict__ fbox;
  const uint32_t* __restrict__ flags;
  const float* __restrict__ rays;
  int64_t n_rays;
  CamArgs cam;
  float iso[8];
  uint32_t iso_on_mask;
  const ViewDesc* views;
  int n_views;
  const int32_t* __restrict__ work;  // queue item -> query index
  RayState* __restrict__ state;
  const RoundPair* __restrict__ pairs;  // element-sorted
  const RoundBatch* __restrict__ batches;
  const unsigned* batch_base;  // this launch's batches: [*batch_base, *batch_base + *n_batches)
  const unsigned* n_batches;
  unsigned* next_batch;
  // mixed-order scenes: element e's record at crec + coff[e] (its own order);
  // coff == nullptr: rec + e * record_floats(N)
  const float* __restrict__ crec;
  const int64_t* __restrict__ coff;
  DevStats* stats;
  // learned mode
  const float* desc;
  const int32_t* cand_e;
  const float* pred;
  unsigned pred_items;
  int warm_cap;  // iterations of a warm-started solve before its cold restart
};

// Task word: kind (3 bits) | pair (5 bits) | argument (8 bits).
enum TaskKind { TK_SAMPLE = 0, TK_REFINE = 1, TK_FSEED = 2, TK_FLEARN = 3, TK_FPOST = 4, TK_IPOST = 5 };
__device__ __forceinline__ uint32_t task_word(int kind, int pp, int arg) {
  return (static_cast<uint32_t>(kind) << 13) | (static_cast<uint32_t>(pp) << 8) | static_cast<uint32_t>(arg);
}

// Per pair, in the warp's shared memory. The sample store is dead once the
// bracket is taken, so the refinement and face-search state overlay it.
struct PairSm {
  float o[3], d[3];
  float te, tx, iso, best_t;
  float pxi[3], pv[3], pk, pte;  // learned prediction (xi at te, d xi/dt per element size)
  int item, elem;
  int fl;        // bit 0 has field, 1 iso on, 2 prediction available, 3 a warm start was rejected
  int pend;      // tasks of the current phase still running
  uint32_t okm;  // samples that converged
  // result under construction
  float ht, hx[3], hg[3];
  int hface;
  int its;  // Newton and face iterations of this pair
  union {
    struct {  // isosurface samples
      float sf[kSamples];
      float sx[kSamples][3];
      // world gradient at each sample, in half precision: only the bracket's
      // left sample's is used, and only as the normal of a hit whose
      // refinement ran out of iterations
      __half sg[kSamples][3];
    };
    struct {
      // refinement
      float rlt, rrt, mt, ct;
      float lsf, lsx[3], lsg[3];
      float rxi[3];
      float msf, msdf, msx[3], msg[3];
      int rit, rstage;
      // face search
      int lf;
      float lt, lx[3];
      int fseed[6];
      float ft[6], fx[6][3];
    };
  };
};

// Rec = false: the tensor-core form keeps the element's coefficients once per
// CTA as its MMA operand instead.
template <int N, bool Rec = true>
struct WarpSm {
  float rec[Rec ? record_floats(N) : 4];
  PairSm pr[RoundCfg<N>::B];
  uint16_t ring[RoundCfg<N>::Ring];
  unsigned head, tail;
  unsigned freem;     // free pair slots
  unsigned admitted;  // pairs of the batch admitted so far
};

template <int N>
constexpr size_t round_smem_bytes() {
  return (kRoundBlock / 32) * ((sizeof(WarpSm<N>) + 15) / 16 * 16);
}

__device__ __forceinline__ float3 ld3(const float* p) { return make_float3(p[0], p[1], p[2]); }
// Warp control words are written by other lanes (plain stores and shared
// atomics) between the warp barriers: always read them from memory.
__device__ __forceinline__ unsigned ld_ctl(const unsigned* p) { return *reinterpret_cast<const volatile unsigned*>(p); }
__device__ __forceinline__ void st3(float* p, float3 v) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
}

// One lane's current solve.
struct LaneSolve {
  int task;  // -1: idle
  int kind, pp, arg;
  float3 xi;  // inverse map: xi; face Newton: the face point
  float t;    // inverse map: the sample's t; face Newton: tau
  int it, cap;
  bool warm, post, inited;
  unsigned tried;  // sample: converged samples of the pair it has restarted from
  float prev;  // face Newton: residual of the last iteration
};

// Every inverse-map iteration of an isosurface solve also evaluates the field
// (value and xi-gradient) at its point. When the step converges (all
// components below 1e-5), the field at the converged point follows from
// these to first order: u(xi - step) = u(xi) - grad u . step, with an error
// of O(|step|^2 |d2u|), below 1e-9 here. The reference evaluates the field
// once more at the converged point instead. A warp pays for its slowest lane,
// and that extra evaluation was one more 4-component step on some lane of
// nearly every warp step; the field's fourth component costs the warp the
// same whether one lane or all evaluate it.

__device__ __forceinline__ void push_task(unsigned* tail, uint16_t* ring, int cap, uint32_t w) {
  const unsigned s = atomicAdd(tail, 1u);
  ring[s % cap] = static_cast<uint16_t>(w);
}

// Start an inverse-map solve of f(t) at t from xi0 (warm: capped, with a cold
// restart on failure).
__device__ __forceinline__ void start_sample_solve(LaneSolve& s, float t, bool warm, float3 xi0, int warm_cap) {
  s.t = t;
  s.warm = warm;
  s.xi = warm ? xi0 : make_float3(0.f, 0.f, 0.f);
  s.it = 0;
  s.cap = warm ? warm_cap : 50;
  s.post = false;
  s.tried = 0u;
}


template <int N>
__device__ __forceinline__ Pred pair_pred(const PairSm& p) {
  Pred pr;
  pr.on = (p.fl & 4) != 0;
  pr.xi_in = ld3(p.pxi);
  pr.v = ld3(p.pv);
  pr.k = p.pk;
  pr.te = p.pte;
  return pr;
}

// A pair is finished: its iterations go to its ray and its slot is free.
template <int N, class WS>
__device__ __forceinline__ void pair_done(WS& W, int pp, const RoundParams* P) {
  const PairSm& p = W.pr[pp];
  atomicAdd(&P->state[p.item].its, p.its);
  atomicOr(&W.freem, 1u << pp);
}

// The pair-level steps below run once per pair phase, not once per Newton
// step, so they are kept out of line: the per-step loop stays small in the
// instruction cache. Counters come back in the return value.

// Queue the 9 seeds of every face (other than the learned face) whose hull
// box meets [0.001, cull_hi]; returns the number of faces culled.
template <int N, class WS>
__device__ __noinline__ int start_seeds(WS* Wp, int pp, const float* __restrict__ fbox, float cull_hi) {
  WS& W = *Wp;
  PairSm& p = W.pr[pp];
  const float3 o = ld3(p.o), d = ld3(p.d);
  int n = 0, culled = 0;
  uint32_t faces = 0;
  for (int f = 0; f < 6; ++f) {
    if (f == p.lf) continue;
    if (face_may_hit(fbox, f, o, d, 0.001f, cull_hi)) {
      faces |= 1u << f;
      n += 9;
    } else {
      ++culled;
    }
  }
  p.pend = n;
  if (n == 0) return culled;
  const unsigned base = atomicAdd(&W.tail, static_cast<unsigned>(n));
  unsigned k = base;
  for (int f = 0; f < 6; ++f)
    if (faces >> f & 1u)
      for (int sd = 0; sd < 9; ++sd)
        W.ring[(k++) % RoundCfg<N>::Ring] = static_cast<uint16_t>(task_word(TK_FSEED, pp, 9 * f + sd));
  return culled;
}

// Nearest face over the learned face and every face's first accepted seed,
// in face order. A hit is left in the pair's result fields (the caller
// starts its post evaluation); no hit finishes the pair.
template <int N, class WS>
__device__ __noinline__ bool finalize_faces(WS* Wp, int pp, const RoundParams* P) {
  WS& W = *Wp;
  PairSm& p = W.pr[pp];
  float best = p.best_t;
  int face = -1;
  float3 xh = make_float3(0.f, 0.f, 0.f);
  for (int f = 0; f < 6; ++f) {
    float tf;
    float3 xf;
    if (f == p.lf) {
      tf = p.lt;
      xf = ld3(p.lx);
    } else if (p.fseed[f] < 9) {
      tf = p.ft[f];
      xf = ld3(p.fx[f]);
    } else {
      continue;
    }
    if (tf > 0.001f && tf < best) {
      best = tf;
      face = f;
      xh = xf;
    }
  }
  if (face < 0) {
    pair_done<N>(W, pp, P);
    return false;
  }
  p.ht = best;
  st3(p.hx, xh);
  p.hface = face;
  return true;
}

__device__ __forceinline__ void start_post(LaneSolve& s, int kind, int pp, float3 xi) {
  s.task = 0;
  s.kind = kind;
  s.pp = pp;
  s.xi = xi;
  s.post = true;
  s.it = 0;
  s.warm = false;
}

// Face search of a pair after its isosurface search found nothing (or iso is
// off): the learned start face first when there is one, else the seeds of
// the faces whose hull box meets [0.001, closest]. Returns culled faces |
// 256 when a learned start was rejected | 65536 when the pair needs its face
// post evaluation now.
template <int N, bool L, class WS>
__device__ __noinline__ int start_faces(WS* Wp, int pp, const float* __restrict__ fbox, const RoundParams* P) {
  WS& W = *Wp;
  PairSm& p = W.pr[pp];
  p.lf = -1;
  for (int f = 0; f < 6; ++f) p.fseed[f] = 9;
  int code = 0;
  if (L && (p.fl & 4)) {
    int f0;
    float3 p0;
    float tau0;
    if (predicted_entry(pair_pred<N>(p), 0.001f, p.best_t, f0, p0, tau0)) {
      p.pend = 1;
      push_task(&W.tail, W.ring, RoundCfg<N>::Ring, task_word(TK_FLEARN, pp, f0));
      return 0;
    }
    code |= 256;
  }
  code |= start_seeds<N>(Wp, pp, fbox, p.best_t);
  if (p.pend == 0 && finalize_faces<N>(Wp, pp, P)) code |= 65536;
  return code;
}

template <int N, bool L, class WS>
__device__ __forceinline__ void face_phase(WS& W, int pp, const float* __restrict__ fbox, const RoundParams* P,
                                           Work& w, LaneSolve& s) {
  const int code = start_faces<N, L>(&W, pp, fbox, P);
  w.culled += code & 255;
  if (code & 256) ++w.rejected;
  if (code & 65536) start_post(s, TK_FPOST, pp, ld3(W.pr[pp].hx));
}

// Begin a popped task.
template <int N, bool L, class WS>
__device__ __forceinline__ void begin_task(WS& W, uint32_t tw, LaneSolve& s, int warm_cap) {
  s.task = static_cast<int>(tw);
  s.kind = static_cast<int>(tw >> 13);
  s.pp = static_cast<int>((tw >> 8) & 31u);
  s.arg = static_cast<int>(tw & 255u);
  if (s.pp >= RoundCfg<N>::B || s.kind > TK_IPOST) {  // never queued: drop it
    s.task = -1;
    return;
  }
  s.inited = false;
  s.prev = FLT_MAX;
  const PairSm& p = W.pr[s.pp];
  if (s.kind == TK_SAMPLE) {
    const float t = p.te + (p.tx - p.te) * (float(s.arg) / 16.0f);
    const bool warm = L && (p.fl & 4);
    start_sample_solve(s, t, warm, warm ? pair_pred<N>(p).at(t) : make_float3(0.f, 0.f, 0.f), warm_cap);
  } else if (s.kind == TK_FSEED) {
    const int f = s.arg / 9, sd = s.arg - 9 * f;
    int fixed, ua, va;
    float val;
    face_param(f, fixed, val, ua, va);
    const int si = sd % 3, sj = sd / 3;
    float3 q = make_float3(0.f, 0.f, 0.f);
    setc(q, fixed, val);
    setc(q, ua, si == 0 ? -0.8f : (si == 1 ? 0.0f : 0.8f));
    setc(q, va, sj == 0 ? -0.8f : (sj == 1 ? 0.0f : 0.8f));
    s.xi = q;
    s.t = 0.f;
    s.it = 0;
    s.cap = 50;
    s.warm = false;
    s.post = false;
  } else {  // TK_FLEARN: the predicted entry face and point
    int f0;
    float3 p0;
    float tau0;
    predicted_entry(pair_pred<N>(p), 0.001f, p.best_t, f0, p0, tau0);
    s.arg = f0;
    s.xi = p0;
    s.t = tau0;
    s.it = 0;
    s.cap = warm_cap;
    s.warm = true;
    s.post = false;
    s.inited = true;
  }
}

// The ray's state after a pair produced a hit.
__device__ __forceinline__ void commit_hit(const RoundParams& P, const PairSm& p, int kind, int face, float t, float3 xi,
                                           float3 n, float u) {
  HitState& b = P.state[p.item].best;
  note_tie(b, p.best_t, t, &P.state[p.item].tie);  // p.best_t: b.t, read when the pair was admitted
  b.t = t;
  b.elem = p.elem;
  b.face = face;
  b.kind = kind;
  b.xi = xi;
  b.n = n;
  b.u = u;
  if (p.fl & 8) b.flags |= HO_FLAG_FALLBACK;
}

// Fill a free slot with a pair of the batch and queue its first tasks.
// Returns start_faces' code for pairs that go straight to the face search.
template <int N, bool L, class WS>
__device__ __noinline__ int admit_pair(WS* Wp, const RoundParams* P, int slot, RoundPair rp, int elem,
                                       bool has_field, const float* __restrict__ fbox) {
  constexpr int R = RoundCfg<N>::Ring;
  WS& W = *Wp;
  PairSm& p = W.pr[slot];
  const int64_t q = P->work[rp.item];
  float3 o, d;
  float iso;
  bool iso_on;
  query_ray_from(P->rays, P->n_rays, P->cam, P->iso, P->iso_on_mask, P->views, P->n_views, q, o, d, iso, iso_on);
  st3(p.o, o);
  st3(p.d, d);
  p.te = rp.te;
  p.tx = rp.tx;
  p.iso = iso;
  p.best_t = P->state[rp.item].best.t;
  p.item = rp.item;
  p.elem = elem;
  int fl = (has_field ? 1 : 0) | (iso_on ? 2 : 0);
  if (L && rp.j >= 0 && rp.j < kPredK && static_cast<unsigned>(rp.item) < P->pred_items &&
      P->cand_e[static_cast<int64_t>(rp.item) * kPredK + rp.j] == elem) {
    const float* y = P->pred + (static_cast<int64_t>(rp.item) * kPredK + rp.j) * kMlpOut;
    p.pxi[0] = y[0]; p.pxi[1] = y[1]; p.pxi[2] = y[2];
    p.pv[0] = y[3]; p.pv[1] = y[4]; p.pv[2] = y[5];
    p.pk = __ldg(P->desc + static_cast<int64_t>(elem) * kDescFloats + 45);
    p.pte = rp.te;
    fl |= 4;
  }
  p.fl = fl;
  p.okm = 0u;
  p.its = 0;
  if ((fl & 3) == 3) {
    p.pend = kSamples;
    const unsigned base = atomicAdd(&W.tail, static_cast<unsigned>(kSamples));
    for (int i = 0; i < kSamples; ++i) W.ring[(base + i) % R] = static_cast<uint16_t>(task_word(TK_SAMPLE, slot, i));
    return 0;
  }
  return start_faces<N, L>(Wp, slot, fbox, P);
}

// Shared memory of the tensor-core form: the CTA's TcSm, then the warps'
// workspaces (no per-warp record).
template <int N, bool TC>
constexpr size_t round_tc_off() {
  return TC ? (sizeof(TcSm) + 127) / 128 * 128 : 0;
}

// TC = false: one warp per element batch, contractions on the CUDA cores from
// the warp's staged record (eval_comps).
// TC = true: one CTA (4 warps) per element batch. Each warp keeps its own pair
// slots and task queue and admits pairs from the CTA's batch; every step the
// 128 threads' points are evaluated together by tcgen05 MMAs against the
// element's coefficients (ho_tc.cuh), so the CTA steps in lockstep: a warp
// with no task joins the step with idle lanes, and the CTA leaves the batch
// when no warp has work and no pair is left.
template <int N, bool L, bool TC>
__global__ void __launch_bounds__(kRoundBlock) round_kernel(RoundParams P) {
  constexpr int B = RoundCfg<N>::B, R = RoundCfg<N>::Ring;
  constexpr unsigned kAllSlots = B >= 32 ? 0xffffffffu : ((1u << B) - 1u);
  constexpr size_t kWarpBytes = (sizeof(WarpSm<N, !TC>) + 15) / 16 * 16;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  extern __shared__ __align__(128) unsigned char round_smem[];
  WarpSm<N, !TC>& W = *reinterpret_cast<WarpSm<N, !TC>*>(round_smem + round_tc_off<N, TC>() + warp * kWarpBytes);
  TcSm& T = *reinterpret_cast<TcSm*>(round_smem);
  Elem<N, true> el;
  el.c = CoefRef<true>{static_cast<uint32_t>(__cvta_generic_to_shared(W.rec))};
  Work w;
  const unsigned nb = *P.n_batches, bbase = *P.batch_base;
  uint32_t tmem = 0, phase = 0;
  bool tc_ok = true;
  if constexpr (TC) {
    if (warp == 0) tc_alloc(&T.tslot);
    if (threadIdx.x == 0) {
      tc_mbar_init(&T.mbar);
      T.ctl[2] = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    tmem = T.tslot;
  }
  for (;;) {
    unsigned b = 0;
    if constexpr (TC) {
      __syncthreads();  // the previous batch is done in every warp
      if (threadIdx.x == 0) {
        T.ctl[0] = atomicAdd(P.next_batch, 1u);
        T.ctl[1] = 0;
      }
      __syncthreads();
      b = T.ctl[0];
    } else {
      if (lane == 0) b = atomicAdd(P.next_batch, 1u);
      b = __shfl_sync(kFull, b, 0);
    }
    if (b >= nb || !tc_ok) break;
    const RoundBatch bt = P.batches[bbase + b];
    const unsigned count = static_cast<unsigned>(bt.count);
    const float* fbox = P.fbox + static_cast<int64_t>(bt.elem) * kFaceBoxFloats;
    {
      const float* recp = P.coff ? P.crec + P.coff[bt.elem] : P.rec + static_cast<int64_t>(bt.elem) * record_floats(N);
      if constexpr (TC) {
        tc_stage_b<N>(T, recp, threadIdx.x, kRoundBlock);
      } else {
        const float4* src = reinterpret_cast<const float4*>(recp);
        float4* dst = reinterpret_cast<float4*>(W.rec);
        for (int q4 = lane; q4 < record_floats(N) / 4; q4 += 32) dst[q4] = __ldg(src + q4);
      }
    }
    const bool has_field = (__ldg(P.flags + bt.elem) & 1u) != 0;
    el.has_field = has_field;
    if (lane == 0) {
      W.head = 0;
      W.tail = 0;
      W.freem = kAllSlots;
      W.admitted = 0;
    }
    if constexpr (TC) {
      tc_proxy_fence();  // the B operand, for the MMAs
      __syncthreads();
    } else {
      __syncwarp();
    }
    LaneSolve s;
    s.task = -1;
    s.kind = 0;
    s.pp = 0;
    s.arg = 0;
    s.xi = make_float3(0.f, 0.f, 0.f);
    s.t = 0.f;
    s.it = 0;
    s.cap = 0;
    s.warm = s.post = s.inited = false;
    s.tried = 0u;
    s.prev = FLT_MAX;
    // every task ends within a bounded number of steps; the guard is far above
    // the longest legal batch and only reports a broken invariant
    for (int guard = 0;; ++guard) {
      if (guard == (1 << 18)) {
        if (lane == 0) atomicOr(&P.stats->status, kStatusRoundGuard);
        break;
      }
      // -- admit the batch's next pairs into free slots
      {
        unsigned fm = 0u, adm = 0u, nadm = 0u;  // lane 0 reads, every lane uses the same values
        if (lane == 0) {
          fm = ld_ctl(&W.freem);
          if constexpr (TC) {  // claim pairs of the CTA's batch for this warp's free slots
            const unsigned want = static_cast<unsigned>(__popc(fm));
            adm = want > 0u && ld_ctl(&T.ctl[1]) < count ? atomicAdd(&T.ctl[1], want) : count;
            nadm = adm < count ? min(want, count - adm) : 0u;
          } else {
            adm = ld_ctl(&W.admitted);
            nadm = min(static_cast<unsigned>(__popc(fm)), count - adm);
          }
        }
        fm = __shfl_sync(kFull, fm, 0);
        adm = __shfl_sync(kFull, adm, 0);
        nadm = __shfl_sync(kFull, nadm, 0);
        __syncwarp();  // every lane has read freem / admitted before any lane changes them
        if (nadm > 0u) {
          if (lane < static_cast<int>(nadm)) {
            unsigned m = fm;  // the lane-th free slot: drop the lowest `lane` set bits
            for (int k = 0; k < lane; ++k) m &= m - 1u;
            const int slot = __ffs(m) - 1;
            if (slot >= 0 && slot < B) {
              atomicAnd(&W.freem, ~(1u << slot));
              const int code = admit_pair<N, L>(&W, &P, slot, P.pairs[bt.first + adm + lane], bt.elem, has_field, fbox);
              ++w.cand;
              w.culled += code & 255;
              if (code & 256) ++w.rejected;  // a face post at admission cannot happen: no face was searched
            } else {
              atomicOr(&P.stats->status, kStatusRoundGuard);
            }
          }
          if (!TC && lane == 0) W.admitted = adm + nadm;
        }
        __syncwarp();
      }
      // -- take tasks
      const unsigned idle = __ballot_sync(kFull, s.task < 0);
      unsigned head = 0u, tail = 0u, admitted = 0u;
      if (lane == 0) {
        head = ld_ctl(&W.head);
        tail = ld_ctl(&W.tail);
        admitted = ld_ctl(&W.admitted);
      }
      head = __shfl_sync(kFull, head, 0);
      tail = __shfl_sync(kFull, tail, 0);
      admitted = __shfl_sync(kFull, admitted, 0);
      unsigned avail = tail - head;
      if constexpr (TC) {
        // a warp whose queue broke its bound stops taking tasks (the status says why)
        if (avail > static_cast<unsigned>(R)) {
          if (lane == 0) atomicOr(&P.stats->status, kStatusRoundGuard);
          avail = 0u;
        }
        const bool warp_busy = !(avail == 0u && idle == kFull);
        const bool more = warp_busy || ld_ctl(&T.ctl[1]) < count;
        if (!__syncthreads_or(lane == 0 && more)) break;  // no warp has work, no pair is left
      } else {
        if (avail > static_cast<unsigned>(R)) {  // the queue can never hold more: a broken invariant
          if (lane == 0) atomicOr(&P.stats->status, kStatusRoundGuard);
          break;
        }
        if (avail == 0u && idle == kFull) {
          if (admitted >= count) break;
          __syncwarp();
          continue;
        }
      }
      const unsigned rank = __popc(idle & ((1u << lane) - 1u));
      if (s.task < 0 && rank < avail) begin_task<N, L>(W, W.ring[(head + rank) % R], s, P.warm_cap);
      __syncwarp();
      if (lane == 0) {
        W.head = head + min(avail, static_cast<unsigned>(__popc(idle)));
        ++w.steps;
        w.lanes += 32u - __popc(idle) + min(avail, static_cast<unsigned>(__popc(idle)));
      }
      // -- evaluate: every busy lane evaluates the geometry at its point
      const bool act = s.task >= 0;
      float3 X = make_float3(0.f, 0.f, 0.f);
      float J[9];
      float u = 0.f;
      float3 gr = make_float3(0.f, 0.f, 0.f);
      // inverse-map iteration of an isosurface solve: the field comes with it
      const bool ahead = (s.kind == TK_SAMPLE || s.kind == TK_REFINE) && !s.post;
      const bool want_geom = act && s.kind != TK_IPOST;
      const bool want_field = act && ((s.post && (s.kind != TK_FPOST || has_field)) || ahead);
      float4 r[4];
      if constexpr (TC) {
        // every thread's point as a row of the step's MMAs; idle lanes give a
        // row at xi = 0 whose results are not used
        const float3 xi = act ? s.xi : make_float3(0.f, 0.f, 0.f);
        float ar[N], dr[N], as[N], ds[N], at[N], dt[N];
        basis_val_der<N>(xi.x, ar, dr);
        basis_val_der<N>(xi.y, as, ds);
        basis_val_der<N>(xi.z, at, dt);
        tc_stage_a<N>(T, threadIdx.x, ar, dr);
        tc_proxy_fence();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (threadIdx.x == 0) tc_issue(T, tmem);
        const bool done = tc_mbar_wait(&T.mbar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!done)) {  // the MMAs did not complete in time: give up the round
          if (threadIdx.x == 0) atomicOr(&P.stats->status, kStatusRoundGuard);
          tc_ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16);
        if (__any_sync(kFull, want_geom)) {
#pragma unroll 1
          for (int comp = 0; comp < 3; ++comp) r[comp] = tc_finish_comp<N>(taddr, comp, as, ds, at, dt);
        }
        if (__any_sync(kFull, want_field)) r[3] = tc_finish_comp<N>(taddr, 3, as, ds, at, dt);
      }
      if (act) {
        if constexpr (!TC) eval_comps<N, true>(el.c, s.xi, want_geom ? 0 : 3, want_field ? 4 : 3, r);
        w.flops += eval_flops(N, (want_geom ? 3 : 0) + (want_field ? 1 : 0));
        if (want_geom) {
          X = make_float3(r[0].x, r[1].x, r[2].x);
          J[0] = r[0].y; J[1] = r[0].z; J[2] = r[0].w;
          J[3] = r[1].y; J[4] = r[1].z; J[5] = r[1].w;
          J[6] = r[2].y; J[7] = r[2].z; J[8] = r[2].w;
          ++w.geom;
        } else {
          for (int q = 0; q < 9; ++q) J[q] = 0.f;
        }
        if (want_field) {
          u = r[3].x;
          gr = make_float3(r[3].y, r[3].z, r[3].w);
          ++w.field;
        }
      }
      // -- advance the solve
      // end: 0 running, 1 converged / accepted, 2 failed
      int end = 0;
      float sf = 0.f, sdf = 0.f;
      float3 sg = make_float3(0.f, 0.f, 0.f);
      if (act) {
        PairSm& p = W.pr[s.pp];
        if (s.kind == TK_SAMPLE || s.kind == TK_REFINE) {
          float K[9];
          invert3(J, K);
          if (!s.post) {
            ++w.newton;
            w.flops += kSolveFlops;
            const float rx = X.x - (p.o[0] + s.t * p.d[0]), ry = X.y - (p.o[1] + s.t * p.d[1]),
                        rz = X.z - (p.o[2] + s.t * p.d[2]);
            const float d0 = K[0] * rx + K[1] * ry + K[2] * rz;
            const float d1 = K[3] * rx + K[4] * ry + K[5] * rz;
            const float d2 = K[6] * rx + K[7] * ry + K[8] * rz;
            s.xi.x -= d0;
            s.xi.y -= d1;
            s.xi.z -= d2;
            ++s.it;
            if (fabsf(d0) < 1e-5f && fabsf(d1) < 1e-5f && fabsf(d2) < 1e-5f) {
              if (ahead) {  // value and gradient at the converged point, first order
                sg = make_float3(K[0] * gr.x + K[3] * gr.y + K[6] * gr.z, K[1] * gr.x + K[4] * gr.y + K[7] * gr.z,
                                 K[2] * gr.x + K[5] * gr.y + K[8] * gr.z);
                sf = (u - (gr.x * d0 + gr.y * d1 + gr.z * d2)) - p.iso;
                sdf = sg.x * p.d[0] + sg.y * p.d[1] + sg.z * p.d[2];
                end = 1;
              } else {
                s.post = true;
              }
            } else if (!(fabsf(d0) + fabsf(d1) + fabsf(d2) < FLT_MAX)) {
              end = 2;
            } else if (s.it >= s.cap) {
              end = 2;
            }
          } else {
            sg = make_float3(K[0] * gr.x + K[3] * gr.y + K[6] * gr.z, K[1] * gr.x + K[4] * gr.y + K[7] * gr.z,
                             K[2] * gr.x + K[5] * gr.y + K[8] * gr.z);
            sf = u - p.iso;
            sdf = sg.x * p.d[0] + sg.y * p.d[1] + sg.z * p.d[2];
            end = 1;
          }
          if (s.warm && end != 0) {
            if (end == 1) {
              ++w.accepted;
            } else {
              ++w.rejected;
              atomicAdd(&p.its, s.it);
              // a sample whose warm start failed starts again from the
              // nearest converged sample of its pair that it has not tried
              // yet (stored in an earlier step), each time capped; when none
              // is left, the plain cold start answers. The cold start is a
              // chain of up to 50 steps that holds its lane and its pair:
              // trying every converged neighbour first took hex64_p5
              // learned from 46.6 to 41.1 ms per call (one neighbour: 46.6;
              // none: 48.6)
              int nb = -1;
              if (s.kind == TK_SAMPLE) {
                int bd = kSamples;
                for (unsigned m = ld_ctl(&p.okm) & ~s.tried; m; m &= m - 1u) {
                  const int j = __ffs(m) - 1, dj = abs(j - s.arg);
                  if (dj < bd) {
                    bd = dj;
                    nb = j;
                  }
                }
              }
              if (nb >= 0) {
                s.tried |= 1u << nb;
                s.xi = ld3(p.sx[nb]);
                s.cap = P.warm_cap;
              } else {
                atomicOr(&p.fl, 8);
                s.warm = false;
                s.xi = make_float3(0.f, 0.f, 0.f);
                s.cap = 50;
              }
              s.it = 0;
              s.post = false;
              end = 0;
            }
          }
        } else if (s.kind == TK_FSEED || s.kind == TK_FLEARN) {
          const int f = s.kind == TK_FSEED ? s.arg / 9 : s.arg;
          int fixed, ua, va;
          float val;
          face_param(f, fixed, val, ua, va);
          const float tmin = 0.001f, tmax = p.best_t;
          if (!s.inited) {  // seed: tau from the seed point's position (same evaluation)
            const float dd = p.d[0] * p.d[0] + p.d[1] * p.d[1] + p.d[2] * p.d[2];
            float tau = dd > 0.f ? ((X.x - p.o[0]) * p.d[0] + (X.y - p.o[1]) * p.d[1] + (X.z - p.o[2]) * p.d[2]) / dd
                                 : 0.f;
            s.t = fminf(fmaxf(tau, tmin), tmax);
            s.inited = true;
          }
          ++w.face;
          w.flops += kSolveFlops;
          const float rx = X.x - (p.o[0] + s.t * p.d[0]), ry = X.y - (p.o[1] + s.t * p.d[1]),
                      rz = X.z - (p.o[2] + s.t * p.d[2]);
          const float m = fmaxf(fabsf(rx), fmaxf(fabsf(ry), fabsf(rz)));
          if (m < 1e-4f) {
            const float pu = getc(s.xi, ua), pv = getc(s.xi, va);
            end = (pu >= -1.001f && pu <= 1.001f && pv >= -1.001f && pv <= 1.001f && s.t >= tmin && s.t <= tmax) ? 1
                                                                                                                : 2;
          } else if (s.it > 5 && m > s.prev * 1.5f) {
            end = 2;
          } else {
            s.prev = m;
            const float A[9] = {J[ua], J[va], -p.d[0], J[3 + ua], J[3 + va], -p.d[1], J[6 + ua], J[6 + va], -p.d[2]};
            float K[9];
            invert3(A, K);
            const float du = -(K[0] * rx + K[1] * ry + K[2] * rz);
            const float dv = -(K[3] * rx + K[4] * ry + K[5] * rz);
            const float dtau = -(K[6] * rx + K[7] * ry + K[8] * rz);
            const float mx = fmaxf(fabsf(du), fmaxf(fabsf(dv), fabsf(dtau)));
            const float sc = mx > 0.25f ? 0.25f / mx : 1.0f;
            float nu = getc(s.xi, ua) + du * sc, nv = getc(s.xi, va) + dv * sc;
            s.t = fminf(fmaxf(s.t + dtau * sc, tmin), tmax);
            nu = fminf(fmaxf(nu, -1.5f), 1.5f);
            nv = fminf(fmaxf(nv, -1.5f), 1.5f);
            setc(s.xi, ua, nu);
            setc(s.xi, va, nv);
            setc(s.xi, fixed, val);
            if (++s.it >= s.cap) end = 2;
          }
          if (end != 0 && s.kind == TK_FLEARN) {
            if (end == 1) ++w.accepted;
            else ++w.rejected;
          }
        } else {
          end = 1;  // post evaluations finish in one step
        }
        if (end != 0) atomicAdd(&p.its, s.it);
      }
      // every lane has read the pair state of this step (the neighbour
      // restart reads the sample store) before any lane writes to it
      __syncwarp();
      // face seeds: the lowest accepted seed index of each face wins
      const bool seed_ok = act && end == 1 && s.kind == TK_FSEED;
      if (seed_ok) atomicMin(&W.pr[s.pp].fseed[s.arg / 9], s.arg % 9);
      if (act && end != 0 && s.kind == TK_SAMPLE) {  // store the sample
        PairSm& p = W.pr[s.pp];
        const int i = s.arg;
        if (end == 1) {
          atomicOr(&p.okm, 1u << i);
          p.sf[i] = sf;
          st3(p.sx[i], s.xi);
          p.sg[i][0] = __float2half_rn(sg.x);
          p.sg[i][1] = __float2half_rn(sg.y);
          p.sg[i][2] = __float2half_rn(sg.z);
        }
      }
      __syncwarp();
      if (seed_ok) {
        PairSm& p = W.pr[s.pp];
        const int f = s.arg / 9;
        if (p.fseed[f] == s.arg % 9) {
          p.ft[f] = s.t;
          st3(p.fx[f], s.xi);
        }
      }
      __syncwarp();
      // -- finished solves: phase transitions
      if (act && end != 0) {
        PairSm& p = W.pr[s.pp];
        const int pp = s.pp;
        const bool warm_pair = L && (p.fl & 4);
        s.task = -1;
        if (s.kind == TK_SAMPLE) {
          if (atomicSub(&p.pend, 1) == 1) {
            // all 17 samples done: first sign change between consecutive good samples
            int prev = -1, found = -1;
            for (int i = 0; i < kSamples; ++i) {
              if (!((p.okm >> i) & 1u)) continue;
              if (prev >= 0 && p.sf[prev] * p.sf[i] <= 0.0f) {
                found = i;
                break;
              }
              prev = i;
            }
            if (found >= 0) {
              // the refinement state overlays the sample store: read first
              const float lf0 = p.sf[prev];
              const float3 lx0 = ld3(p.sx[prev]), rx0 = ld3(p.sx[found]);
              const float3 lg0 = make_float3(__half2float(p.sg[prev][0]), __half2float(p.sg[prev][1]),
                                             __half2float(p.sg[prev][2]));
              p.rlt = p.te + (p.tx - p.te) * (float(prev) / 16.0f);
              p.rrt = p.te + (p.tx - p.te) * (float(found) / 16.0f);
              p.lsf = lf0;
              st3(p.lsx, lx0);
              st3(p.lsg, lg0);
              st3(p.rxi, rx0);
              p.rit = 0;
              p.rstage = 0;
              p.mt = 0.5f * (p.rlt + p.rrt);
              s.task = 0;
              s.kind = TK_REFINE;
              s.pp = pp;
              start_sample_solve(s, p.mt, warm_pair, lerp3(ld3(p.lsx), ld3(p.rxi), 0.5f), P.warm_cap);
            } else {
              face_phase<N, L>(W, pp, fbox, &P, w, s);
            }
          }
        } else if (s.kind == TK_REFINE) {
          if (p.rstage == 0) {  // midpoint solve ended
            if (end == 2) {
              face_phase<N, L>(W, pp, fbox, &P, w, s);  // the isosurface search failed
            } else {
              p.msf = sf;
              p.msdf = sdf;
              st3(p.msx, s.xi);
              st3(p.msg, sg);
              float ct = p.mt;
              if (fabsf(sdf) > 1e-8f) {
                const float nt = p.mt - sf / sdf;
                if (nt > p.rlt && nt < p.rrt) ct = nt;
              }
              p.ct = ct;
              p.rstage = 1;
              s.task = 0;
              start_sample_solve(s, ct, warm_pair, s.xi, P.warm_cap);
            }
          } else {  // Newton candidate solve ended
            float ct = p.ct, csf;
            float3 csx = s.xi, csg;
            if (end == 1) {
              csf = sf;
              csg = sg;
            } else {  // keep the failed solve's xi
              ct = p.mt;
              csf = p.msf;
              csg = ld3(p.msg);
            }
            bool found = false;
            if (fabsf(csf) < 1e-5f) {
              p.ht = ct;
              st3(p.hx, csx);
              st3(p.hg, csg);
              found = true;
            } else {
              if (p.lsf * csf <= 0.0f) {
                p.rrt = ct;
                st3(p.rxi, csx);
              } else {
                p.rlt = ct;
                p.lsf = csf;
                st3(p.lsx, csx);
                st3(p.lsg, csg);
              }
              if (++p.rit >= 20) {
                p.ht = 0.5f * (p.rlt + p.rrt);
                for (int c = 0; c < 3; ++c) {
                  p.hx[c] = p.lsx[c];
                  p.hg[c] = p.lsg[c];
                }
                found = true;
              } else {
                p.mt = 0.5f * (p.rlt + p.rrt);
                p.rstage = 0;
                s.task = 0;
                start_sample_solve(s, p.mt, warm_pair, lerp3(ld3(p.lsx), ld3(p.rxi), 0.5f), P.warm_cap);
              }
            }
            if (found) {  // the field value at the root's xi, then the hit
              s.task = 0;
              s.kind = TK_IPOST;
              s.xi = ld3(p.hx);
              s.post = true;
              s.it = 0;
              s.warm = false;
            }
          }
        } else if (s.kind == TK_FSEED) {
          if (atomicSub(&p.pend, 1) == 1 && finalize_faces<N>(&W, pp, &P)) start_post(s, TK_FPOST, pp, ld3(p.hx));
        } else if (s.kind == TK_FLEARN) {
          if (end == 1) {
            p.lf = s.arg;
            p.lt = s.t;
            st3(p.lx, s.xi);
          }
          w.culled += start_seeds<N>(&W, pp, fbox, end == 1 ? s.t : p.best_t);
          if (p.pend == 0 && finalize_faces<N>(&W, pp, &P)) start_post(s, TK_FPOST, pp, ld3(p.hx));
        } else if (s.kind == TK_FPOST) {
          // normal from the Jacobian columns (the face's two tangents)
          const float3 dr = make_float3(J[0], J[3], J[6]), ds = make_float3(J[1], J[4], J[7]),
                       dt = make_float3(J[2], J[5], J[8]);
          const float3 xi = s.xi;
          float3 n;
          if (fabsf(xi.x) > 0.9f) n = cross3(ds, dt);
          else if (fabsf(xi.y) > 0.9f) n = cross3(dr, dt);
          else n = cross3(dr, ds);
          n = normalize3(n);
          if (n.x * p.d[0] + n.y * p.d[1] + n.z * p.d[2] > 0.f) n = make_float3(-n.x, -n.y, -n.z);
          commit_hit(P, p, HO_HIT_FACE, p.hface, p.ht, xi, n, has_field ? u : 0.f);
          pair_done<N>(W, pp, &P);
        } else if (s.kind == TK_IPOST) {
          if (p.ht > 0.001f && p.ht < p.best_t) {
            float3 n = normalize3(ld3(p.hg));
            if (n.x * p.d[0] + n.y * p.d[1] + n.z * p.d[2] > 0.f) n = make_float3(-n.x, -n.y, -n.z);
            commit_hit(P, p, HO_HIT_ISO, -1, p.ht, s.xi, n, u);
          }
          pair_done<N>(W, pp, &P);
        }
      }
      __syncwarp();
    }
  }
  if constexpr (TC) {
    // MMAs still in flight after a timed-out wait complete before the
    // accumulator columns are freed (bounded again)
    if (!tc_ok && threadIdx.x == 0) tc_mbar_wait(&T.mbar, phase ^ 1u);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem);
  }
  flush_work(P.stats, w, false);
}

// The tail: rays still in flight after the main rounds, each finished by one
// warp that walks the rest of its ordered candidates (the warp-per-ray form
// of the same per-candidate solves, visit_warp). A round lasts as long as its
// slowest pair, so the last rounds, with few pairs each, wait mostly on
// chains of refinement and face solves; here every ray proceeds at its own
// pace. Elements are staged at the scene's largest order (padded records).
template <int N, bool L>
__global__ void __launch_bounds__(kTraceBlock) tail_kernel(TraceParams P, RayState* __restrict__ st,
                                                           const uint32_t* __restrict__ list,
                                                           const unsigned* __restrict__ n_list,
                                                           unsigned* __restrict__ next) {
  const int lane = threadIdx.x & 31;
  extern __shared__ __align__(16) float tail_stage[];
  float4* slot4 = reinterpret_cast<float4*>(tail_stage + (threadIdx.x >> 5) * record_floats(N));
  const uint32_t slot_addr = static_cast<uint32_t>(__cvta_generic_to_shared(slot4));
  Work w, wu;
  const unsigned n = *n_list;
  for (;;) {
    unsigned k = 0;
    if (lane == 0) k = atomicAdd(next, 1u);
    k = __shfl_sync(kFull, k, 0);
    if (k >= n) break;
    const unsigned item = list[k];
    RayState& r = st[item];
    float3 o, d;
    float iso;
    bool iso_on;
    query_ray(P, P.work[item], o, d, iso, iso_on);
    HitState best = r.best;
    float kt = r.kt;
    int ke = r.ke, pass = r.pass, first = r.cursor;
    bool overflow = r.ovf != 0;
    // this ray's iterations: the warp's (per-lane w summed, wu once) now less
    // at the start
    uint32_t w0 = w.newton + w.face;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) w0 += __shfl_xor_sync(kFull, w0, off);
    const uint32_t it0 = wu.newton + wu.face + w0;
    float bt[kCandK];
    int be[kCandK];
    const float2* kb = P.kbuf + static_cast<int64_t>(item) * kCandK;
#pragma unroll
    for (int j = 0; j < kCandK; ++j) {
      const float2 c = kb[j];
      bt[j] = c.x;
      be[j] = __float_as_int(c.y);
    }
    for (int guard = 0; guard < (1 << 20); ++guard) {
      bool done = false;
#pragma unroll 1
      for (int j = first; j < kCandK; ++j) {
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
          const float4* src = reinterpret_cast<const float4*>(P.rec + static_cast<int64_t>(ce) * record_floats(N));
          __syncwarp();
          for (int q4 = lane; q4 < record_floats(N) / 4; q4 += 32) slot4[q4] = __ldg(src + q4);
          __syncwarp();
          Elem<N, true> el;
          el.c = CoefRef<true>{slot_addr};
          el.has_field = (__ldg(P.flags + ce) & 1u) != 0;
          Pred pr;
          pr.on = false;
          if (L && pass == 0 && j < kPredK && item < P.pred_items &&
              P.cand_e[static_cast<int64_t>(item) * kPredK + j] == ce) {
            const float* y = P.pred + (static_cast<int64_t>(item) * kPredK + j) * kMlpOut;
            pr.on = true;
            pr.xi_in = make_float3(y[0], y[1], y[2]);
            pr.v = make_float3(y[3], y[4], y[5]);
            pr.k = __ldg(P.desc + static_cast<int64_t>(ce) * kDescFloats + 45);
            pr.te = te;
          }
          visit_warp<N, L>(el, P.fbox + static_cast<int64_t>(ce) * kFaceBoxFloats, ce, o, d, te, tx, iso, iso_on,
                           best, w, wu, pr, &r.tie);
        }
        kt = ct;
        ke = ce;
      }
      if (done || !overflow) break;
      // the list was cut at kCandK: walk the tree again after the last visited key
      if (!collect(P, o, d, best.t, kt, ke, bt, be, overflow, wu)) {
        if (lane == 0) atomicOr(&P.stats->status, kStatusStackOverflow);
        best.flags |= HO_FLAG_INCOMPLETE;
        break;
      }
      first = 0;
      ++pass;
      ++wu.restarts;
      best.flags |= HO_FLAG_OVERFLOW;
    }
    uint32_t its = w.newton + w.face;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) its += __shfl_xor_sync(kFull, its, off);
    __syncwarp();
    if (lane == 0) {
      r.best = best;
      r.its += static_cast<int>(its + wu.newton + wu.face - it0);
      r.done = 1;
    }
  }
  if (lane == 0) {
    w.cand += wu.cand; w.geom += wu.geom; w.map += wu.map; w.field += wu.field; w.newton += wu.newton;
    w.face += wu.face; w.culled += wu.culled; w.nodes += wu.nodes; w.restarts += wu.restarts;
    w.accepted += wu.accepted; w.rejected += wu.rejected;
  }
  w.flops = 0;  // the flop counter describes the round kernel only
  flush_work(P.stats, w, false);
}

template <int N>
cudaError_t launch_tail_n(const TraceParams& P, RayState* st, const uint32_t* list, const unsigned* n_list,
                          unsigned* next, bool learned, cudaStream_t s) {
  // persistent grid per device and form (kernel attributes are set per
  // device); two host threads that fill the same entry at once store the same
  // value
  static std::atomic<int> grid[kGridCacheDevices][2];
  const size_t smem = static_cast<size_t>(kTraceBlock / 32) * record_floats(N) * sizeof(float);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kGridCacheDevices) return cudaErrorInvalidDevice;
  int g = grid[dev][learned ? 1 : 0].load(std::memory_order_acquire);
  if (g == 0) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (learned) {
      cudaFuncSetAttribute(tail_kernel<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tail_kernel<N, true>, kTraceBlock, smem);
    } else {
      cudaFuncSetAttribute(tail_kernel<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tail_kernel<N, false>, kTraceBlock, smem);
    }
    g = sms * (per > 0 ? per : 1);
    grid[dev][learned ? 1 : 0].store(g, std::memory_order_release);
  }
  if (learned) tail_kernel<N, true><<<g, kTraceBlock, smem, s>>>(P, st, list, n_list, next);
  else tail_kernel<N, false><<<g, kTraceBlock, smem, s>>>(P, st, list, n_list, next);
  return cudaGetLastError();
}

template <int N, bool L, bool TC>
static cudaError_t launch_round_kernel(const RoundParams& R, cudaStream_t s) {
  // persistent grid: resident blocks per SM x SMs (the tensor-core form holds
  // all of an SM's tensor memory, so one CTA per SM: its shared memory request
  // is raised to more than half of the SM's)
  // per device (kernel attributes are set per device); two host threads that
  // fill the same entry at once store the same values. The grid is stored
  // last (release) and read first (acquire), so a thread that sees it sees
  // the shared-memory size and the attribute set before it.
  static std::atomic<int> grid[kGridCacheDevices];
  static std::atomic<int> smem_of[kGridCacheDevices];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kGridCacheDevices) return cudaErrorInvalidDevice;
  int g = grid[dev].load(std::memory_order_acquire);
  size_t smem = static_cast<size_t>(smem_of[dev].load(std::memory_order_relaxed));
  if (g == 0) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    smem = round_tc_off<N, TC>() + (kRoundBlock / 32) * ((sizeof(WarpSm<N, !TC>) + 15) / 16 * 16);
    if (TC) {
      int max_optin = 0;
      cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      smem = std::max<size_t>(smem, static_cast<size_t>(max_optin) / 2 + 1024);
    }
    cudaFuncSetAttribute(round_kernel<N, L, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, round_kernel<N, L, TC>, kRoundBlock, smem);
    g = sms * (TC ? 1 : (per > 0 ? per : 1));
    smem_of[dev].store(static_cast<int>(smem), std::memory_order_relaxed);
    grid[dev].store(g, std::memory_order_release);
  }
  round_kernel<N, L, TC><<<g, kRoundBlock, smem, s>>>(R);
  return cudaGetLastError();
}

// tc: the tensor-core form (orders up to kTcMaxModes).
template <int N>
cudaError_t launch_round_n(const RoundParams& R, cudaStream_t s, bool learned, bool tc) {
  if constexpr (N <= kTcMaxModes) {
    if (tc) return learned ? launch_round_kernel<N, true, true>(R, s) : launch_round_kernel<N, false, true>(R, s);
  }
  return learned ? launch_round_kernel<N, true, false>(R, s) : launch_round_kernel<N, false, false>(R, s);
}

// explicit instantiations live in ho_trace_n*.cu
extern template cudaError_t launch_round_n<2>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
extern template cudaError_t launch_round_n<3>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
extern template cudaError_t launch_round_n<4>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
extern template cudaError_t launch_round_n<5>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
extern template cudaError_t launch_round_n<6>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
extern template cudaError_t launch_round_n<7>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
extern template cudaError_t launch_round_n<8>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);
extern template cudaError_t launch_round_n<9>(const RoundParams& R, cudaStream_t s, bool learned, bool tc);

extern template cudaError_t launch_tail_n<2>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);
extern template cudaError_t launch_tail_n<3>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);
extern template cudaError_t launch_tail_n<4>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);
extern template cudaError_t launch_tail_n<5>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);
extern template cudaError_t launch_tail_n<6>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);
extern template cudaError_t launch_tail_n<7>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);
extern template cudaError_t launch_tail_n<8>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);
extern template cudaError_t launch_tail_n<9>(const TraceParams&, RayState*, const uint32_t*, const unsigned*, unsigned*,
                                             bool, cudaStream_t);

}  // namespace ho
