// Data layouts shared by host code and kernels.
#pragma once

#include <cstdint>

#include "horender.h"

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#endif
#endif

namespace ho {

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
  ST_COUNT
};

struct DevStats {
  unsigned long long c[ST_COUNT];
  int status;  // nonzero: a kernel met an internal limit (see kStatus*)
  int pad[3];
};

constexpr int kStatusStackOverflow = 1;
constexpr int kStatusBadModes = 2;

// Per-face hull boxes: 6 faces x (lo xyz, hi xyz).
constexpr int kFaceBoxFloats = 36;

// Largest supported modes per direction (P = 8).
constexpr int kMaxModes = 9;
constexpr int kMinModes = 2;

}  // namespace ho
