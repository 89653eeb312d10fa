// Data layouts shared by host code and kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "horender.h"

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#endif
#endif

namespace ho {

// Pinhole camera of one view: pixel (x, y) looks along
// llc + s*horiz + t*vert - origin, s = (x + 0.5)/full_w, t = (y + 0.5)/full_h.
// A call covers the width x height pixels starting at (x0, y0) of the
// full_w x full_h image (the whole image: x0 = y0 = 0, full = width, height).
struct CamArgs {
  float3 origin, llc, horiz, vert;
  int width, height;
  int x0, y0, full_w, full_h;
};

// One camera view of a multi-view call: its pixel-centre rays are queries
// [q0, q0 + width * height * n_iso), isovalue-major like a single view.
struct ViewDesc {
  CamArgs cam;
  int64_t q0;
  int n_iso;
  uint32_t iso_on_mask;
  float iso[8];
};

// BVH child record: the child's box plus its index. idx >= 0: internal node;
// idx < 0: leaf holding element ~idx; idx == kEmptyChild: unused slot.
// aux carries leaf flags (bit 0: element has a field).
struct alignas(16) ChildRec {
  float lo[3];
  int32_t idx;
  float hi[3];
  uint32_t aux;
};

// Internal node = the two child records (64 bytes, one 64-B line: each child
// is one 32-B sector, fetched as two float4).
struct alignas(64) BNode {
  ChildRec c[2];
};

constexpr int32_t kEmptyChild = INT32_MIN;
constexpr uint32_t kAuxHasField = 1u;

// Device counters (one slot per ho_stats field that kernels update).
enum StatSlot {
  ST_RAYS = 0,
  ST_CAND,
  ST_GEOM,
  ST_MAP,
  ST_FIELD,
  ST_NEWTON,
  ST_FACE,
  ST_CULLED,
  ST_NODES,
  ST_ACCEPT,
  ST_REJECT,
  ST_RESTART,
  ST_CYC_TRAV,
  ST_CYC_SCAN,
  ST_CYC_REFINE,
  ST_CYC_FACE,
  ST_STEPS,
  ST_LANES,
  ST_ROUNDS,
  ST_PAIRS,
  ST_CHECKED,
  ST_CHECK_FAIL,
  ST_CHECK_FINAL,
  ST_FLOPS,
  ST_TAIL,
  ST_FLUSH,  // the slots before this one are summed by the hexahedron kernels' flush
  ST_PRIM_CAND = ST_FLUSH,
  ST_PRIM_ITERS,
  ST_PRIM_FLOPS,
  ST_PRIM_NODES,
  ST_POLISHED,  // hits refined by the FP64 polish (check and plain kernels)
  ST_TIES,      // rays with a tie partner that the FP64 tie rule weighed
  ST_TIES_SWAPPED,  // of those, rays whose partner won
  ST_GRAZING,       // hits with |cos| between ray and surface below kGrazeCos
  ST_COUNT
};

struct DevStats {
  unsigned long long c[ST_COUNT];
  int status;  // nonzero: a kernel met an internal limit (see kStatus*)
  int pad[3];
};

constexpr int kStatusStackOverflow = 1;
constexpr int kStatusBadModes = 2;
constexpr int kStatusRoundGuard = 4;

// Per-face hull boxes: 6 faces x (lo xyz, hi xyz).
constexpr int kFaceBoxFloats = 36;

// Largest supported modes per direction (P = 8).
constexpr int kMaxModes = 9;
// Pair slots per warp of the round kernel: the per-warp shared memory (element
// record, pair slots, task queue) is sized so that three 4-warp blocks fit on
// an SM up to N = 8 (two at N = 9, whose record alone is 15.5 KB).
constexpr int round_slots(int n) { return n <= 7 ? 20 : (n == 8 ? 12 : 8); }
// The round kernel's tensor-core form takes orders up to this (N*N <= 64
// accumulator columns per component); one CTA of 4 warps per element batch.
constexpr int kTcMaxModes = 8;
// Default pairs per element batch: a warp's slots, or a CTA's with tc.
__host__ __device__ constexpr int round_batch_default(int n, bool tc) {
  return tc && n <= kTcMaxModes ? 4 * round_slots(n) : round_slots(n);
}
constexpr int kMinModes = 2;

// Element record layout: x, y, z geometry blocks then the field block; in a
// block, coefficient (i,j,k) sits at (k*N + j)*RS + i with the row stride RS
// = N rounded up to a multiple of 4 (rows start on 16-byte boundaries, so a
// row is fetched with float4 loads; the padding is zero).
__host__ __device__ constexpr int row_stride(int n) { return (n + 3) & ~3; }
__host__ __device__ constexpr int block_floats(int n) { return n * n * row_stride(n); }
__host__ __device__ constexpr int record_floats(int n) { return 4 * block_floats(n); }

}  // namespace ho
