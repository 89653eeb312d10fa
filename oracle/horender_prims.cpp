// C entry points of the primitive oracle (TEST INFRASTRUCTURE ONLY; see
// horender_prims.hpp). Built into the same library as horender_oracle.cpp.
//
// Scene input mirrors the reference's Scene::add_prism / add_quad /
// add_curved_tri (FEM-AABB/raytracer.h:167-300) as one list: per primitive its
// kind, vertices (6 / 4 / 3 used), modes, an offset into one flat geometry
// array (x, y, z blocks, each as long as the kind's block; -1 = linear) and
// into one flat field array (-1 = no field).
//
// Tracing order (the product's): the hexahedra are traced first; the
// primitives are then visited in ascending (box entry t, list index) order,
// each clipped to the closest hit so far, which starts at the hexahedra's
// hit. The reference visits hexes and primitives together in BVH stack
// order instead.
#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "horender_prims.hpp"

using namespace horacle;

extern "C" {

typedef struct {
  int32_t n;
  const int32_t* kind;          // n: 0 prism, 1 quad, 2 triangle
  const float* verts;           // n x 6 x 3
  const uint32_t* geom_modes;   // n x 3
  const int64_t* geom_offset;   // n, -1 => linear
  const float* geom;
  int64_t geom_len;
  const uint32_t* field_modes;  // n x 3
  const int64_t* field_offset;  // n, -1 => no field
  const float* field;
  int64_t field_len;
} hor_prims_desc;

// Same record as horender_oracle.cpp's.
typedef struct {
  double t;
  int32_t elem, face, kind, pad;
  double xi[3];
  double n[3];
  double u;
} hor_prim_hit;
}

namespace {

constexpr int kHitPrism = 3;  // hit kinds of the three primitive kinds: 3 + kind

struct GNode {
  double lo[3], hi[3];
  int left, right;  // leaf: left = first in `order`, right = -count - 1
};

struct PScene {
  std::vector<float> geom, field;
  std::vector<Prim> prims;
  std::vector<int> local;  // index among the primitives of the same kind
  std::vector<double> box32, box64;
  // candidate gathering: a median-split tree over boxes holding both
  // precisions' boxes, slightly inflated; the exact test decides afterwards
  std::vector<double> gbox;
  std::vector<int> order;
  std::vector<GNode> nodes;
};

int build_gather(PScene& s, int first, int count) {
  GNode nd;
  for (int a = 0; a < 3; ++a) {
    nd.lo[a] = 1e300;
    nd.hi[a] = -1e300;
  }
  for (int i = 0; i < count; ++i) {
    const double* b = &s.gbox[6 * s.order[first + i]];
    for (int a = 0; a < 3; ++a) {
      nd.lo[a] = std::min(nd.lo[a], b[a]);
      nd.hi[a] = std::max(nd.hi[a], b[3 + a]);
    }
  }
  const int me = static_cast<int>(s.nodes.size());
  s.nodes.push_back(nd);
  if (count <= 4) {
    s.nodes[me].left = first;
    s.nodes[me].right = -count - 1;
    return me;
  }
  int axis = 0;
  for (int a = 1; a < 3; ++a)
    if (nd.hi[a] - nd.lo[a] > nd.hi[axis] - nd.lo[axis]) axis = a;
  const int mid = first + count / 2;
  std::nth_element(s.order.begin() + first, s.order.begin() + mid, s.order.begin() + first + count,
                   [&](int x, int y) {
                     const double cx = s.gbox[6 * x + axis] + s.gbox[6 * x + 3 + axis];
                     const double cy = s.gbox[6 * y + axis] + s.gbox[6 * y + 3 + axis];
                     return cx < cy || (cx == cy && x < y);
                   });
  const int l = build_gather(s, first, mid - first);
  const int r = build_gather(s, mid, first + count - mid);
  s.nodes[me].left = l;
  s.nodes[me].right = r;
  return me;
}

bool slab_line(const double* lo, const double* hi, const double o[3], const double d[3]) {
  double te = 0.0, tx = 1e300;
  for (int a = 0; a < 3; ++a) {
    if (std::fabs(d[a]) < 1e-12) {
      if (o[a] < lo[a] || o[a] > hi[a]) return false;
      continue;
    }
    double t0 = (lo[a] - o[a]) / d[a], t1 = (hi[a] - o[a]) / d[a];
    if (t0 > t1) std::swap(t0, t1);
    te = std::max(te, t0);
    tx = std::min(tx, t1);
    if (te > tx) return false;
  }
  return true;
}

// Every primitive whose inflated box the ray's half-line meets.
void gather(const PScene& s, const float* rf, std::vector<int>& out) {
  out.clear();
  if (s.nodes.empty()) return;
  const double o[3] = {rf[0], rf[1], rf[2]}, d[3] = {rf[3], rf[4], rf[5]};
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const GNode& n = s.nodes[stack[--sp]];
    if (!slab_line(n.lo, n.hi, o, d)) continue;
    if (n.right < 0) {
      for (int i = 0; i < -n.right - 1; ++i) out.push_back(s.order[n.left + i]);
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.right;
    }
  }
}

template <class R> void boxes(const PScene& s, std::vector<double>& out) {
  out.assign(s.prims.size() * 6, 0.0);
  for (size_t i = 0; i < s.prims.size(); ++i) {
    R lo[3], hi[3];
    prim_box<R>(s.prims[i], lo, hi);
    for (int a = 0; a < 3; ++a) {
      out[6 * i + a] = static_cast<double>(lo[a]);
      out[6 * i + 3 + a] = static_cast<double>(hi[a]);
    }
  }
}

template <class R> void box_of(const PScene& s, int i, R lo[3], R hi[3]) {
  const std::vector<double>& b = sizeof(R) == sizeof(float) ? s.box32 : s.box64;
  for (int a = 0; a < 3; ++a) {
    lo[a] = static_cast<R>(b[6 * i + a]);
    hi[a] = static_cast<R>(b[6 * i + 3 + a]);
  }
}

template <class R> void trace_one(const PScene& s, const float* rf, hor_prim_hit& io,
                                  std::vector<std::pair<R, int>>& cands, std::vector<int>& near) {
  Ray<R> ray;
  ray.o = mk<R>(rf[0], rf[1], rf[2]);
  ray.d = mk<R>(rf[3], rf[4], rf[5]);
  const R eps = static_cast<R>(0.001f);
  R best = io.kind != 0 ? static_cast<R>(io.t) : static_cast<R>(FLT_MAX);
  cands.clear();
  gather(s, rf, near);
  for (int i : near) {
    R lo[3], hi[3], te, tx;
    box_of<R>(s, i, lo, hi);
    if (ray_box<R>(ray, mk<R>(lo[0], lo[1], lo[2]), mk<R>(hi[0], hi[1], hi[2]), eps, best, te, tx))
      cands.push_back({te, i});
  }
  std::sort(cands.begin(), cands.end());
  for (const auto& c : cands) {
    if (c.first > best) break;
    const int i = c.second;
    R lo[3], hi[3], te, tx;
    box_of<R>(s, i, lo, hi);
    if (!ray_box<R>(ray, mk<R>(lo[0], lo[1], lo[2]), mk<R>(hi[0], hi[1], hi[2]), eps, best, te, tx)) continue;
    R t;
    V3<R> x;
    if (!prim_intersect<R>(s.prims[i], lo, hi, ray, eps, best, t, x)) continue;
    if (!(t > eps && t < best)) continue;
    best = t;
    const Prim& p = s.prims[i];
    const V3<R> n = prim_normal<R>(p, x, ray.d);
    io.t = static_cast<double>(t);
    io.elem = s.local[i];
    io.face = -1;
    io.kind = kHitPrism + p.kind;
    io.xi[0] = x.x; io.xi[1] = x.y; io.xi[2] = x.z;
    io.n[0] = n.x; io.n[1] = n.y; io.n[2] = n.z;
    io.u = static_cast<double>(prim_field<R>(p, x));
  }
}

template <class F> void parallel_for(int64_t n, int nthreads, F&& fn) {
  if (nthreads <= 1 || n < 64) {
    fn(0, n);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> pool;
  for (int w = 0; w < nthreads; ++w)
    pool.emplace_back([&] {
      for (;;) {
        const int64_t b = next.fetch_add(16);
        if (b >= n) break;
        fn(b, std::min(n, b + 16));
      }
    });
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {

void* hor_prims_create(const hor_prims_desc* d) {
  PScene* s = new PScene();
  s->geom.assign(d->geom, d->geom + d->geom_len);
  s->field.assign(d->field, d->field + d->field_len);
  int count[3] = {0, 0, 0};
  for (int i = 0; i < d->n; ++i) {
    Prim p;
    std::memset(&p, 0, sizeof(p));
    p.kind = d->kind[i];
    for (int v = 0; v < 6; ++v)
      for (int a = 0; a < 3; ++a) p.verts[v][a] = d->verts[(6 * i + v) * 3 + a];
    for (int a = 0; a < 3; ++a) {
      p.gm[a] = d->geom_modes[3 * i + a];
      p.fm[a] = d->field_modes[3 * i + a];
    }
    if (d->geom_offset[i] >= 0) {
      const int64_t blk = prim_block_size(p.kind, p.gm);
      for (int a = 0; a < 3; ++a) p.geom[a] = s->geom.data() + d->geom_offset[i] + a * blk;
    } else {
      p.gm[0] = p.gm[1] = p.gm[2] = 0;
    }
    p.field = d->field_offset[i] >= 0 ? s->field.data() + d->field_offset[i] : nullptr;
    s->prims.push_back(p);
    s->local.push_back(count[p.kind]++);
  }
  boxes<float>(*s, s->box32);
  boxes<double>(*s, s->box64);
  const int n = static_cast<int>(s->prims.size());
  s->gbox.resize(6 * static_cast<size_t>(n));
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      const double lo = std::min(s->box32[6 * i + a], s->box64[6 * i + a]);
      const double hi = std::max(s->box32[6 * i + 3 + a], s->box64[6 * i + 3 + a]);
      s->gbox[6 * i + a] = lo - 1e-6 * (1.0 + std::fabs(lo));
      s->gbox[6 * i + 3 + a] = hi + 1e-6 * (1.0 + std::fabs(hi));
    }
  s->order.resize(n);
  for (int i = 0; i < n; ++i) s->order[i] = i;
  if (n > 0) build_gather(*s, 0, n);
  return s;
}

void hor_prims_destroy(void* s) { delete static_cast<PScene*>(s); }

int hor_prims_boxes(void* sp, int precision, double* out) {
  PScene* s = static_cast<PScene*>(sp);
  const std::vector<double>& b = precision == 32 ? s->box32 : s->box64;
  std::memcpy(out, b.data(), b.size() * sizeof(double));
  return 0;
}

// One primitive against n rays on given segments [seg[2i], seg[2i+1]]:
// out[5i..5i+4] = (hit 0/1, t, r, s, t-coordinate).
int hor_prims_intersect(void* sp, int precision, int prim, const float* rays, int64_t n, const double* seg,
                        double* out) {
  PScene* s = static_cast<PScene*>(sp);
  if (prim < 0 || prim >= static_cast<int>(s->prims.size())) return -1;
  const Prim& p = s->prims[prim];
  for (int64_t i = 0; i < n; ++i) {
    const float* rf = rays + 6 * i;
    double* o = out + 5 * i;
    std::fill(o, o + 5, 0.0);
    if (precision == 32) {
      Ray<float> ray{mk<float>(rf[0], rf[1], rf[2]), mk<float>(rf[3], rf[4], rf[5])};
      float lo[3], hi[3], t;
      V3<float> x;
      box_of<float>(*s, prim, lo, hi);
      if (prim_intersect<float>(p, lo, hi, ray, static_cast<float>(seg[2 * i]), static_cast<float>(seg[2 * i + 1]), t,
                                x)) {
        o[0] = 1;
        o[1] = t; o[2] = x.x; o[3] = x.y; o[4] = x.z;
      }
    } else {
      Ray<double> ray{mk<double>(rf[0], rf[1], rf[2]), mk<double>(rf[3], rf[4], rf[5])};
      double lo[3], hi[3], t;
      V3<double> x;
      box_of<double>(*s, prim, lo, hi);
      if (prim_intersect<double>(p, lo, hi, ray, seg[2 * i], seg[2 * i + 1], t, x)) {
        o[0] = 1;
        o[1] = t; o[2] = x.x; o[3] = x.y; o[4] = x.z;
      }
    }
  }
  return 0;
}

// Map points: out[3i..3i+2] = x(xi_i) of primitive `prim`.
int hor_prims_map(void* sp, int precision, int prim, const double* xi, int64_t n, double* out) {
  PScene* s = static_cast<PScene*>(sp);
  if (prim < 0 || prim >= static_cast<int>(s->prims.size())) return -1;
  for (int64_t i = 0; i < n; ++i) {
    if (precision == 32) {
      const V3<float> x = prim_map<float>(s->prims[prim], mk<float>(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]));
      out[3 * i] = x.x; out[3 * i + 1] = x.y; out[3 * i + 2] = x.z;
    } else {
      const V3<double> x = prim_map<double>(s->prims[prim], mk<double>(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]));
      out[3 * i] = x.x; out[3 * i + 1] = x.y; out[3 * i + 2] = x.z;
    }
  }
  return 0;
}

// Primitive pass after the hexahedra: io holds each ray's hexahedron hit
// (kind 0 = miss) and receives the merged answer.
int hor_prims_trace(void* sp, int precision, const float* rays, int64_t n, hor_prim_hit* io, int nthreads) {
  PScene* s = static_cast<PScene*>(sp);
  parallel_for(n, nthreads, [&](int64_t b, int64_t e) {
    std::vector<int> near;
    if (precision == 32) {
      std::vector<std::pair<float, int>> c;
      for (int64_t i = b; i < e; ++i) trace_one<float>(*s, rays + 6 * i, io[i], c, near);
    } else {
      std::vector<std::pair<double, int>> c;
      for (int64_t i = b; i < e; ++i) trace_one<double>(*s, rays + 6 * i, io[i], c, near);
    }
  });
  return 0;
}
}
