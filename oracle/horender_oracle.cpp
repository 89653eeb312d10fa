// C entry points of the CPU oracle (TEST INFRASTRUCTURE ONLY; see
// horender_oracle.hpp). Built into oracle/_build/libhorender_oracle.so by
// oracle/Makefile with -ffp-contract=off so FP32 results do not depend on
// whether the host compiler fuses multiply-adds.
//
// Scene input mirrors what the reference's Scene::add_hex stores
// (FEM-AABB/raytracer.h:118-166): per element the modes, an offset into one
// flat geometry array (x, y, z blocks of nx*ny*nz floats each) and an offset
// into one flat field array (-1 = no field), plus the 8 corner vertices.
#include <atomic>
#include <cstring>
#include <thread>

#include "horender_oracle.hpp"

using namespace horacle;

extern "C" {

typedef struct {
  int32_t n_elem;
  const uint32_t* geom_modes;   // n_elem x 3
  const int64_t* geom_offset;   // n_elem, -1 => trilinear
  const float* geom;
  const uint32_t* field_modes;  // n_elem x 3
  const int64_t* field_offset;  // n_elem, -1 => no field
  const float* field;
  const float* verts;           // n_elem x 8 x 3
} hor_scene_desc;

typedef struct {
  double t;
  int32_t elem, face, kind, pad;
  double xi[3];
  double n[3];
  double u;
} hor_hit;

typedef struct {
  uint64_t newton_iters, face_iters, newton_solves, candidates;
} hor_counters;
}

namespace {

struct Box64 {
  double lo[3], hi[3];
};

struct GatherNode {
  Box64 b;
  int left, right;  // leaf: left = first, right = -count-1
};

struct OScene {
  std::vector<Elem> elems;
  std::vector<Box64> box32, box64;  // padded sampled boxes in f32 / f64 (computed on first use)
  std::vector<uint8_t> have_box;
  std::vector<Box64> gbox;          // cheap rigorous superset of both, for candidate gathering
  std::vector<GatherNode> nodes;
  std::vector<int> order;
};

// A box that contains the padded sampled box without sampling: the vertex
// modes (i,j,k in {0,1}) interpolate trilinearly between 8 values, and every
// other mode is bounded by |phi_i| <= (i-1)/4 on [-1,1] (|P^{(1,1)}_m| <= m+1
// there); the result is then padded the way the sampled box is.
Box64 gather_box(const Elem& e) {
  Box64 b;
  if (!has_ho_geom(e)) {
    for (int a = 0; a < 3; ++a) {
      b.lo[a] = 1e300;
      b.hi[a] = -1e300;
      for (int v = 0; v < 8; ++v) {
        b.lo[a] = std::min(b.lo[a], double(e.verts[v][a]));
        b.hi[a] = std::max(b.hi[a], double(e.verts[v][a]));
      }
      b.lo[a] -= 1e-4 + 1e-6;
      b.hi[a] += 1e-4 + 1e-6;
    }
    return b;
  }
  auto bound = [](unsigned i) { return i < 2 ? 1.0 : 0.25 * (double(i) - 1.0); };
  for (int a = 0; a < 3; ++a) {
    const float* c = e.geom[a];
    double lo = 1e300, hi = -1e300, rest = 0.0;
    int idx = 0;
    for (unsigned k = 0; k < e.gm[2]; ++k)
      for (unsigned j = 0; j < e.gm[1]; ++j)
        for (unsigned i = 0; i < e.gm[0]; ++i) {
          const double v = c[idx++];
          if (i < 2 && j < 2 && k < 2) {
            lo = std::min(lo, v);
            hi = std::max(hi, v);
          } else {
            rest += std::fabs(v) * bound(i) * bound(j) * bound(k);
          }
        }
    lo -= rest;
    hi += rest;
    const double pad = std::max(0.15 * (hi - lo), 1e-3) * 1.001 + 1e-6 * (1.0 + std::fabs(lo) + std::fabs(hi));
    b.lo[a] = lo - pad;
    b.hi[a] = hi + pad;
  }
  return b;
}

void compute_boxes(OScene& s, int64_t i) {
  V3<float> l32, h32;
  V3<double> l64, h64;
  elem_box<float>(s.elems[i], 4, l32, h32);
  elem_box<double>(s.elems[i], 4, l64, h64);
  Box64& a = s.box32[i];
  Box64& c = s.box64[i];
  a.lo[0] = l32.x; a.lo[1] = l32.y; a.lo[2] = l32.z; a.hi[0] = h32.x; a.hi[1] = h32.y; a.hi[2] = h32.z;
  c.lo[0] = l64.x; c.lo[1] = l64.y; c.lo[2] = l64.z; c.hi[0] = h64.x; c.hi[1] = h64.y; c.hi[2] = h64.z;
  s.have_box[i] = 1;
}

int build_gather(OScene& s, int first, int count) {
  GatherNode nd;
  Box64 b;
  for (int a = 0; a < 3; ++a) { b.lo[a] = 1e300; b.hi[a] = -1e300; }
  for (int i = 0; i < count; ++i) {
    const Box64& c = s.gbox[s.order[first + i]];
    for (int a = 0; a < 3; ++a) { b.lo[a] = std::min(b.lo[a], c.lo[a]); b.hi[a] = std::max(b.hi[a], c.hi[a]); }
  }
  nd.b = b;
  const int me = static_cast<int>(s.nodes.size());
  s.nodes.push_back(nd);
  if (count <= 4) {
    s.nodes[me].left = first;
    s.nodes[me].right = -count - 1;
    return me;
  }
  int axis = 0;
  double ext = -1;
  for (int a = 0; a < 3; ++a)
    if (b.hi[a] - b.lo[a] > ext) { ext = b.hi[a] - b.lo[a]; axis = a; }
  const int mid = first + count / 2;
  std::nth_element(s.order.begin() + first, s.order.begin() + mid, s.order.begin() + first + count,
                   [&](int x, int y) {
                     const double cx = s.gbox[x].lo[axis] + s.gbox[x].hi[axis];
                     const double cy = s.gbox[y].lo[axis] + s.gbox[y].hi[axis];
                     return cx < cy || (cx == cy && x < y);
                   });
  const int l = build_gather(s, first, mid - first);
  const int r = build_gather(s, mid, first + count - mid);
  s.nodes[me].left = l;
  s.nodes[me].right = r;
  return me;
}

bool slab64(const Box64& b, const double o[3], const double d[3]) {
  double te = 0.0, tx = 1e300;
  for (int a = 0; a < 3; ++a) {
    if (std::fabs(d[a]) < 1e-12) {
      if (o[a] < b.lo[a] || o[a] > b.hi[a]) return false;
      continue;
    }
    double t0 = (b.lo[a] - o[a]) / d[a], t1 = (b.hi[a] - o[a]) / d[a];
    if (t0 > t1) std::swap(t0, t1);
    te = std::max(te, t0);
    tx = std::min(tx, t1);
    if (te > tx) return false;
  }
  return true;
}

// Every element whose (slightly inflated) box the ray line touches for t >= 0.
void gather(const OScene& s, const double o[3], const double d[3], std::vector<int>& out) {
  out.clear();
  if (s.nodes.empty()) return;
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const GatherNode& n = s.nodes[stack[--sp]];
    if (!slab64(n.b, o, d)) continue;
    if (n.right < 0) {
      const int cnt = -n.right - 1;
      for (int i = 0; i < cnt; ++i) out.push_back(s.order[n.left + i]);
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.right;
    }
  }
}

template <class R>
void trace_one(const OScene& s, const float* rayf, float isof, bool iso_on, hor_hit& out, Counters& cnt,
               uint64_t& ncand, const std::vector<int>& scratch, std::vector<std::pair<R, int>>& cands) {
  Ray<R> ray;
  ray.o = mk<R>(rayf[0], rayf[1], rayf[2]);
  ray.d = mk<R>(rayf[3], rayf[4], rayf[5]);
  const std::vector<Box64>& boxes = (sizeof(R) == sizeof(float)) ? s.box32 : s.box64;
  const R t_eps = static_cast<R>(0.001f);
  const R t_far = static_cast<R>(FLT_MAX);
  cands.clear();
  for (int e : scratch) {
    const Box64& b = boxes[e];
    const V3<R> lo = mk<R>(static_cast<R>(b.lo[0]), static_cast<R>(b.lo[1]), static_cast<R>(b.lo[2]));
    const V3<R> hi = mk<R>(static_cast<R>(b.hi[0]), static_cast<R>(b.hi[1]), static_cast<R>(b.hi[2]));
    R te, tx;
    if (ray_box<R>(ray, lo, hi, t_eps, t_far, te, tx)) cands.push_back({te, e});
  }
  std::sort(cands.begin(), cands.end());
  Hit<R> best;
  best.t = t_far;
  best.elem = -1;
  best.face = -1;
  best.kind = HK_MISS;
  best.xi = mk<R>(0, 0, 0);
  best.n = mk<R>(0, 0, 0);
  best.u = 0;
  for (const auto& c : cands) {
    if (c.first > best.t) break;
    const int e = c.second;
    const Box64& b = boxes[e];
    const V3<R> lo = mk<R>(static_cast<R>(b.lo[0]), static_cast<R>(b.lo[1]), static_cast<R>(b.lo[2]));
    const V3<R> hi = mk<R>(static_cast<R>(b.hi[0]), static_cast<R>(b.hi[1]), static_cast<R>(b.hi[2]));
    R te, tx;
    if (!ray_box<R>(ray, lo, hi, t_eps, best.t, te, tx)) continue;
    ++ncand;
    visit_candidate<R>(s.elems[e], e, ray, te, tx, static_cast<R>(isof), iso_on, best, &cnt);
  }
  out.t = static_cast<double>(best.t);
  out.elem = best.elem;
  out.face = best.face;
  out.kind = best.kind;
  out.pad = 0;
  out.xi[0] = best.xi.x; out.xi[1] = best.xi.y; out.xi[2] = best.xi.z;
  out.n[0] = best.n.x; out.n[1] = best.n.y; out.n[2] = best.n.z;
  out.u = static_cast<double>(best.u);
}

template <class F>
void parallel_for(int64_t n, int nthreads, F&& fn) {
  if (nthreads <= 1 || n < 64) {
    fn(0, 0, n);
    return;
  }
  std::atomic<int64_t> next{0};
  const int64_t chunk = 16;
  std::vector<std::thread> pool;
  for (int w = 0; w < nthreads; ++w) {
    pool.emplace_back([&, w] {
      for (;;) {
        const int64_t b = next.fetch_add(chunk);
        if (b >= n) break;
        fn(w, b, std::min(n, b + chunk));
      }
    });
  }
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {

void* hor_scene_create(const hor_scene_desc* d) {
  OScene* s = new OScene();
  s->elems.resize(d->n_elem);
  for (int i = 0; i < d->n_elem; ++i) {
    Elem& e = s->elems[i];
    std::memset(&e, 0, sizeof(e));
    for (int a = 0; a < 3; ++a) {
      e.gm[a] = d->geom_modes[3 * i + a];
      e.fm[a] = d->field_modes[3 * i + a];
    }
    if (d->geom_offset[i] >= 0) {
      const int64_t cnt = static_cast<int64_t>(e.gm[0]) * e.gm[1] * e.gm[2];
      for (int a = 0; a < 3; ++a) e.geom[a] = d->geom + d->geom_offset[i] + a * cnt;
    } else {
      e.gm[0] = e.gm[1] = e.gm[2] = 0;
    }
    e.field = d->field_offset[i] >= 0 ? d->field + d->field_offset[i] : nullptr;
    for (int v = 0; v < 8; ++v)
      for (int a = 0; a < 3; ++a) e.verts[v][a] = d->verts[(i * 8 + v) * 3 + a];
  }
  s->box32.resize(d->n_elem);
  s->box64.resize(d->n_elem);
  s->have_box.assign(d->n_elem, 0);
  s->gbox.resize(d->n_elem);
  parallel_for(d->n_elem, std::max(1u, std::thread::hardware_concurrency()), [&](int, int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) s->gbox[i] = gather_box(s->elems[i]);
  });
  s->order.resize(d->n_elem);
  for (int i = 0; i < d->n_elem; ++i) s->order[i] = i;
  if (d->n_elem > 0) build_gather(*s, 0, d->n_elem);
  return s;
}

void hor_scene_destroy(void* s) { delete static_cast<OScene*>(s); }

// Padded sampled boxes as (lo.xyz, hi.xyz) per element, in f32 or f64 math.
int hor_scene_boxes(void* sp, int precision, double* out) {
  OScene* s = static_cast<OScene*>(sp);
  parallel_for(static_cast<int64_t>(s->elems.size()), std::max(1u, std::thread::hardware_concurrency()),
               [&](int, int64_t b, int64_t e) {
                 for (int64_t i = b; i < e; ++i)
                   if (!s->have_box[i]) compute_boxes(*s, i);
               });
  const std::vector<Box64>& b = precision == 32 ? s->box32 : s->box64;
  for (size_t i = 0; i < b.size(); ++i)
    for (int a = 0; a < 3; ++a) {
      out[6 * i + a] = b[i].lo[a];
      out[6 * i + 3 + a] = b[i].hi[a];
    }
  return 0;
}

// Trace n rays (6 floats each: origin, direction). iso_on = 0 disables the
// isosurface (the reference disables it when iso == 0, raytracer.cu:207; the
// caller decides). precision: 32 or 64.
int hor_trace(void* sp, int precision, const float* rays, int64_t n, float iso, int iso_on, int nthreads,
              hor_hit* out, hor_counters* counters) {
  OScene* s = static_cast<OScene*>(sp);
  std::vector<hor_counters> per(std::max(1, nthreads));
  for (auto& c : per) std::memset(&c, 0, sizeof(c));
  // 1. candidates per ray through the rigorous gather boxes
  std::vector<std::vector<int>> lists(n);
  parallel_for(n, nthreads, [&](int, int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const float* r = rays + 6 * i;
      const double o64[3] = {r[0], r[1], r[2]}, d64[3] = {r[3], r[4], r[5]};
      gather(*s, o64, d64, lists[i]);
    }
  });
  // 2. exact padded boxes for the touched elements
  std::vector<int> need;
  {
    std::vector<uint8_t> mark(s->elems.size(), 0);
    for (const auto& l : lists)
      for (int e : l)
        if (!s->have_box[e] && !mark[e]) {
          mark[e] = 1;
          need.push_back(e);
        }
  }
  parallel_for(static_cast<int64_t>(need.size()), nthreads, [&](int, int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) compute_boxes(*s, need[i]);
  });
  // 3. trace
  parallel_for(n, nthreads, [&](int w, int64_t b, int64_t e) {
    Counters cnt;
    uint64_t ncand = 0;
    if (precision == 32) {
      std::vector<std::pair<float, int>> cands;
      for (int64_t i = b; i < e; ++i) trace_one<float>(*s, rays + 6 * i, iso, iso_on != 0, out[i], cnt, ncand, lists[i], cands);
    } else {
      std::vector<std::pair<double, int>> cands;
      for (int64_t i = b; i < e; ++i) trace_one<double>(*s, rays + 6 * i, iso, iso_on != 0, out[i], cnt, ncand, lists[i], cands);
    }
    per[w].newton_iters += cnt.newton_iters;
    per[w].face_iters += cnt.face_iters;
    per[w].newton_solves += cnt.newton_solves;
    per[w].candidates += ncand;
  });
  if (counters) {
    std::memset(counters, 0, sizeof(*counters));
    for (auto& c : per) {
      counters->newton_iters += c.newton_iters;
      counters->face_iters += c.face_iters;
      counters->newton_solves += c.newton_solves;
      counters->candidates += c.candidates;
    }
  }
  return 0;
}

// Replay a given candidate visit order (e.g. recorded from the reference's
// own BVH walk) with the same per-candidate policy: each listed element is
// box-tested against [0.001, closest] and visited if it passes. Isolates the
// per-candidate policy from the traversal order.
int hor_trace_replay(void* sp, int precision, const float* rays, int64_t n, float iso, int iso_on,
                     const int32_t* order, int order_cap, const int32_t* order_n, hor_hit* out) {
  OScene* s = static_cast<OScene*>(sp);
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < std::min(order_cap, order_n[i]); ++k)
      if (!s->have_box[order[i * order_cap + k]]) compute_boxes(*s, order[i * order_cap + k]);
  for (int64_t i = 0; i < n; ++i) {
    const int m = std::min(order_cap, order_n[i]);
    Counters cnt;
    auto run = [&](auto tag) {
      using R = decltype(tag);
      const float* rf = rays + 6 * i;
      Ray<R> ray{mk<R>(rf[0], rf[1], rf[2]), mk<R>(rf[3], rf[4], rf[5])};
      const std::vector<Box64>& boxes = (sizeof(R) == sizeof(float)) ? s->box32 : s->box64;
      Hit<R> best;
      best.t = static_cast<R>(FLT_MAX);
      best.elem = -1; best.face = -1; best.kind = HK_MISS;
      best.xi = mk<R>(0, 0, 0); best.n = mk<R>(0, 0, 0); best.u = 0;
      for (int k = 0; k < m; ++k) {
        const int e = order[i * order_cap + k];
        const Box64& b = boxes[e];
        const V3<R> lo = mk<R>(static_cast<R>(b.lo[0]), static_cast<R>(b.lo[1]), static_cast<R>(b.lo[2]));
        const V3<R> hi = mk<R>(static_cast<R>(b.hi[0]), static_cast<R>(b.hi[1]), static_cast<R>(b.hi[2]));
        R te, tx;
        if (!ray_box<R>(ray, lo, hi, static_cast<R>(0.001f), best.t, te, tx)) continue;
        visit_candidate<R>(s->elems[e], e, ray, te, tx, static_cast<R>(iso), iso_on != 0, best, &cnt);
      }
      hor_hit& o = out[i];
      o.t = static_cast<double>(best.t); o.elem = best.elem; o.face = best.face; o.kind = best.kind; o.pad = 0;
      o.xi[0] = best.xi.x; o.xi[1] = best.xi.y; o.xi[2] = best.xi.z;
      o.n[0] = best.n.x; o.n[1] = best.n.y; o.n[2] = best.n.z;
      o.u = static_cast<double>(best.u);
    };
    if (precision == 32) run(float{});
    else run(double{});
  }
  return 0;
}

// ---- the judge's polish ------------------------------------------------------
// FP64 Newton on the equations that define a hit, from the hit's own (t, xi),
// iterated to convergence: a face hit on face f solves x(xi) = o + t d with
// xi's fixed coordinate held at the face value (unknowns: the two free
// coordinates and t); an isosurface hit solves x(xi) = o + t d and
// u(xi) = iso (unknowns: xi and t). The reference's own stopping rules
// (face residual below 1e-4, |u - iso| below 1e-5) leave t uncertain by up
// to their tolerances; the polished hit is the exact root of the same
// equations near the returned one, the yardstick for the error of every
// hit. hits: in/out (HIT_DTYPE); pad = 1 when the iteration converged (t
// step below 1e-13 relative, xi steps below 1e-10), 0 otherwise (the hit is
// left as it was).
int hor_polish(void* sp, const float* rays, int64_t n, float isof, hor_hit* hits, int nthreads) {
  OScene* s = static_cast<OScene*>(sp);
  parallel_for(n, nthreads, [&](int, int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      hor_hit& h = hits[i];
      h.pad = 0;
      if ((h.kind != HK_FACE && h.kind != HK_ISO) || h.elem < 0) continue;
      const Elem& el = s->elems[h.elem];
      const double o[3] = {rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]};
      const double d[3] = {rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]};
      V3<double> xi = mk<double>(h.xi[0], h.xi[1], h.xi[2]);
      double t = h.t;
      const bool iso_hit = h.kind == HK_ISO;
      if (iso_hit && !el.field) continue;
      FaceParam fp{};
      if (!iso_hit) fp = face_param(h.face);
      bool ok = false;
      for (int it = 0; it < 30; ++it) {
        const V3<double> x = map_point<double>(el, xi);
        double J[9];
        jacobian<double>(el, xi, J);
        const double r[3] = {x.x - (o[0] + t * d[0]), x.y - (o[1] + t * d[1]), x.z - (o[2] + t * d[2])};
        double dx[3] = {0, 0, 0}, dt = 0;
        if (iso_hit) {
          double K[9];
          invert3<double>(J, K);
          const V3<double> g = field_grad_ref<double>(el, xi);
          const double f = field_value<double>(el, xi) - static_cast<double>(isof);
          double a[3], bb[3];
          for (int k = 0; k < 3; ++k) {
            a[k] = -(K[3 * k] * r[0] + K[3 * k + 1] * r[1] + K[3 * k + 2] * r[2]);
            bb[k] = K[3 * k] * d[0] + K[3 * k + 1] * d[1] + K[3 * k + 2] * d[2];
          }
          const double gb = g.x * bb[0] + g.y * bb[1] + g.z * bb[2];
          if (gb == 0.0) break;
          dt = (-f - (g.x * a[0] + g.y * a[1] + g.z * a[2])) / gb;
          for (int k = 0; k < 3; ++k) dx[k] = a[k] + bb[k] * dt;
        } else {
          // columns: d x / d xi_u, d x / d xi_v, -d
          const double A[9] = {J[fp.u], J[fp.v], -d[0], J[3 + fp.u], J[3 + fp.v], -d[1], J[6 + fp.u], J[6 + fp.v],
                               -d[2]};
          double K[9];
          invert3<double>(A, K);
          const double du = -(K[0] * r[0] + K[1] * r[1] + K[2] * r[2]);
          const double dv = -(K[3] * r[0] + K[4] * r[1] + K[5] * r[2]);
          dt = -(K[6] * r[0] + K[7] * r[1] + K[8] * r[2]);
          dx[fp.u] = du;
          dx[fp.v] = dv;
        }
        if (!(std::isfinite(dx[0]) && std::isfinite(dx[1]) && std::isfinite(dx[2]) && std::isfinite(dt))) break;
        xi = mk<double>(xi.x + dx[0], xi.y + dx[1], xi.z + dx[2]);
        t += dt;
        const double mx = std::fmax(std::fabs(dx[0]), std::fmax(std::fabs(dx[1]), std::fabs(dx[2])));
        if (mx > 0.05 || std::fabs(dt) > 0.05) break;  // walked away from the returned hit: not its root
        // xi steps are world steps over |J| (about h/2), so xi settles at a
        // coarser level than t
        if (std::fabs(dt) < 1e-13 * std::fmax(1.0, std::fabs(t)) && mx < 1e-10) {
          ok = true;
          break;
        }
      }
      if (!ok) continue;
      h.pad = 1;
      h.t = t;
      h.xi[0] = xi.x;
      h.xi[1] = xi.y;
      h.xi[2] = xi.z;
      h.u = el.field ? field_value<double>(el, xi) : 0.0;
    }
  });
  return 0;
}

// ---- element-level entry points (known-answer tests) ----------------------

int hor_map_point(void* sp, int precision, int elem, const double* xi, int64_t n, double* out_x) {
  const OScene* s = static_cast<const OScene*>(sp);
  const Elem& e = s->elems[elem];
  for (int64_t i = 0; i < n; ++i) {
    if (precision == 32) {
      V3<float> p = map_point<float>(e, mk<float>(float(xi[3 * i]), float(xi[3 * i + 1]), float(xi[3 * i + 2])));
      out_x[3 * i] = p.x; out_x[3 * i + 1] = p.y; out_x[3 * i + 2] = p.z;
    } else {
      V3<double> p = map_point<double>(e, mk<double>(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]));
      out_x[3 * i] = p.x; out_x[3 * i + 1] = p.y; out_x[3 * i + 2] = p.z;
    }
  }
  return 0;
}

// out: 9 Jacobian entries + field value + 3 world-gradient entries per point.
int hor_eval_point(void* sp, int precision, int elem, const double* xi, int64_t n, double* out) {
  const OScene* s = static_cast<const OScene*>(sp);
  const Elem& e = s->elems[elem];
  for (int64_t i = 0; i < n; ++i) {
    double* o = out + 13 * i;
    if (precision == 32) {
      const V3<float> p = mk<float>(float(xi[3 * i]), float(xi[3 * i + 1]), float(xi[3 * i + 2]));
      float J[9];
      jacobian<float>(e, p, J);
      for (int k = 0; k < 9; ++k) o[k] = J[k];
      o[9] = e.field ? field_value<float>(e, p) : 0.f;
      V3<float> g = e.field ? field_grad_world<float>(e, p) : mk<float>(0, 0, 0);
      o[10] = g.x; o[11] = g.y; o[12] = g.z;
    } else {
      const V3<double> p = mk<double>(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]);
      double J[9];
      jacobian<double>(e, p, J);
      for (int k = 0; k < 9; ++k) o[k] = J[k];
      o[9] = e.field ? field_value<double>(e, p) : 0.0;
      V3<double> g = e.field ? field_grad_world<double>(e, p) : mk<double>(0, 0, 0);
      o[10] = g.x; o[11] = g.y; o[12] = g.z;
    }
  }
  return 0;
}

// Inverse map from xi = 0; out per point: xi (3) + converged flag.
int hor_inverse_map(void* sp, int precision, int elem, const double* x, int64_t n, double* out) {
  const OScene* s = static_cast<const OScene*>(sp);
  const Elem& e = s->elems[elem];
  for (int64_t i = 0; i < n; ++i) {
    double* o = out + 4 * i;
    if (precision == 32) {
      V3<float> xi;
      const bool ok = inverse_map<float>(e, mk<float>(float(x[3 * i]), float(x[3 * i + 1]), float(x[3 * i + 2])), xi, nullptr);
      o[0] = xi.x; o[1] = xi.y; o[2] = xi.z; o[3] = ok ? 1.0 : 0.0;
    } else {
      V3<double> xi;
      const bool ok = inverse_map<double>(e, mk<double>(x[3 * i], x[3 * i + 1], x[3 * i + 2]), xi, nullptr);
      o[0] = xi.x; o[1] = xi.y; o[2] = xi.z; o[3] = ok ? 1.0 : 0.0;
    }
  }
  return 0;
}

// Isosurface search on [t0,t1]; out per ray: found, t, xi(3), grad(3).
int hor_find_iso(void* sp, int precision, int elem, const float* rays, const double* seg, int64_t n, float iso,
                 double* out) {
  const OScene* s = static_cast<const OScene*>(sp);
  const Elem& e = s->elems[elem];
  for (int64_t i = 0; i < n; ++i) {
    double* o = out + 8 * i;
    const float* r = rays + 6 * i;
    if (precision == 32) {
      Ray<float> ray{mk<float>(r[0], r[1], r[2]), mk<float>(r[3], r[4], r[5])};
      float th = 0; V3<float> xi = mk<float>(0, 0, 0), g = mk<float>(0, 0, 0);
      const bool ok = find_iso<float>(e, ray, float(seg[2 * i]), float(seg[2 * i + 1]), iso, th, xi, g, nullptr);
      o[0] = ok; o[1] = th; o[2] = xi.x; o[3] = xi.y; o[4] = xi.z; o[5] = g.x; o[6] = g.y; o[7] = g.z;
    } else {
      Ray<double> ray{mk<double>(r[0], r[1], r[2]), mk<double>(r[3], r[4], r[5])};
      double th = 0; V3<double> xi = mk<double>(0, 0, 0), g = mk<double>(0, 0, 0);
      const bool ok = find_iso<double>(e, ray, seg[2 * i], seg[2 * i + 1], double(iso), th, xi, g, nullptr);
      o[0] = ok; o[1] = th; o[2] = xi.x; o[3] = xi.y; o[4] = xi.z; o[5] = g.x; o[6] = g.y; o[7] = g.z;
    }
  }
  return 0;
}

// Nearest curved-face hit in [tmin,tmax]; out per ray: hit, t, xi(3), face.
int hor_hit_hex(void* sp, int precision, int elem, const float* rays, const double* seg, int64_t n, double* out) {
  const OScene* s = static_cast<const OScene*>(sp);
  const Elem& e = s->elems[elem];
  for (int64_t i = 0; i < n; ++i) {
    double* o = out + 6 * i;
    const float* r = rays + 6 * i;
    int face = -1;
    if (precision == 32) {
      Ray<float> ray{mk<float>(r[0], r[1], r[2]), mk<float>(r[3], r[4], r[5])};
      float th = 0; V3<float> xi = mk<float>(0, 0, 0);
      const bool ok = hit_hex<float>(e, ray, float(seg[2 * i]), float(seg[2 * i + 1]), th, xi, face, nullptr);
      o[0] = ok; o[1] = th; o[2] = xi.x; o[3] = xi.y; o[4] = xi.z; o[5] = face;
    } else {
      Ray<double> ray{mk<double>(r[0], r[1], r[2]), mk<double>(r[3], r[4], r[5])};
      double th = 0; V3<double> xi = mk<double>(0, 0, 0);
      const bool ok = hit_hex<double>(e, ray, seg[2 * i], seg[2 * i + 1], th, xi, face, nullptr);
      o[0] = ok; o[1] = th; o[2] = xi.x; o[3] = xi.y; o[4] = xi.z; o[5] = face;
    }
  }
  return 0;
}

// Basis values for a KAT: out[2*i] = ModifiedA(i,x), out[2*i+1] = derivative.
int hor_basis(int precision, unsigned nmodes, double x, double* out) {
  for (unsigned i = 0; i < nmodes; ++i) {
    if (precision == 32) {
      out[2 * i] = mod_a<float>(i, float(x));
      out[2 * i + 1] = mod_a_prime<float>(i, float(x));
    } else {
      out[2 * i] = mod_a<double>(i, x);
      out[2 * i + 1] = mod_a_prime<double>(i, x);
    }
  }
  return 0;
}

// Pinhole camera rays (FEM-AABB/raytracer.h:31-48 with aperture 0) through
// pixel centres, row y = 0 at the bottom of the view; 6 floats per ray.
int hor_camera_rays(const float* from, const float* at, const float* vup, float vfov_deg, int W, int H, float* out) {
  const float theta = vfov_deg * 3.14159265f / 180.0f;
  const float h = std::tan(theta / 2.0f);
  const float vh = 2.0f * h, vw = (float(W) / float(H)) * vh;
  V3<float> w = mk<float>(from[0] - at[0], from[1] - at[1], from[2] - at[2]);
  const float focus = std::sqrt(dot3(w, w));
  w = normalize3(w);
  V3<float> u = normalize3(cross3(mk<float>(vup[0], vup[1], vup[2]), w));
  V3<float> v = cross3(w, u);
  const V3<float> hor = mk<float>(focus * vw * u.x, focus * vw * u.y, focus * vw * u.z);
  const V3<float> ver = mk<float>(focus * vh * v.x, focus * vh * v.y, focus * vh * v.z);
  const V3<float> llc = mk<float>(from[0] - hor.x / 2.0f - ver.x / 2.0f - focus * w.x,
                                  from[1] - hor.y / 2.0f - ver.y / 2.0f - focus * w.y,
                                  from[2] - hor.z / 2.0f - ver.z / 2.0f - focus * w.z);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const float s = (float(x) + 0.5f) / float(W), t = (float(y) + 0.5f) / float(H);
      V3<float> d = mk<float>(llc.x + s * hor.x + t * ver.x - from[0], llc.y + s * hor.y + t * ver.y - from[1],
                              llc.z + s * hor.z + t * ver.z - from[2]);
      d = normalize3(d);
      float* o = out + 6 * (static_cast<int64_t>(y) * W + x);
      o[0] = from[0]; o[1] = from[1]; o[2] = from[2];
      o[3] = d.x; o[4] = d.y; o[5] = d.z;
    }
  return 0;
}

// Primary-ray shading: Lambert headlight on hits (material 1 = blue on face
// 0, else grey, as raytracer.cu:247-248 assigns), sky gradient on misses
// (raytracer.cu:398-402), gamma 2 and 8-bit quantisation
// (raytracer.cu:462-475). out: 3 bytes per ray.
int hor_shade(const float* rays, const hor_hit* hits, int64_t n, uint8_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    const float* r = rays + 6 * i;
    float c[3];
    if (hits[i].kind == HK_MISS) {
      const float a = 0.5f * (r[4] + 1.0f);
      c[0] = (1.0f - a) * 1.0f + a * 0.5f;
      c[1] = (1.0f - a) * 1.0f + a * 0.7f;
      c[2] = (1.0f - a) * 1.0f + a * 1.0f;
    } else {
      const bool blue = hits[i].kind == HK_FACE && hits[i].face == 0;
      const float alb[3] = {blue ? 0.1f : 0.5f, blue ? 0.2f : 0.5f, blue ? 0.8f : 0.5f};
      float lam = -(float(hits[i].n[0]) * r[3] + float(hits[i].n[1]) * r[4] + float(hits[i].n[2]) * r[5]);
      lam = lam > 0.f ? lam : 0.f;
      for (int k = 0; k < 3; ++k) c[k] = alb[k] * (0.2f + 0.8f * lam);
    }
    for (int k = 0; k < 3; ++k) {
      const float g = std::fmin(1.0f, std::sqrt(c[k]));
      out[3 * i + k] = static_cast<uint8_t>(255.99f * g);
    }
  }
  return 0;
}

}  // extern "C"
