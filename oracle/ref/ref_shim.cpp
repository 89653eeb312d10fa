// Thin C shim over the reference's own host code, used ONLY to pin the
// oracle and to generate golden vectors (TEST INFRASTRUCTURE). It is compiled
// together with the reference sources, where they lie, by oracle/build_ref.sh
// into oracle/_ref/libref.so; nothing here is shipped or linked by the
// product.
//
// Everything numeric is done by the reference's functions; this file only
// marshals arrays. The one piece the reference has only in device code is its
// traversal, bvh_intersect_device (FEM-AABB/raytracer.cu:102-358); ref_trace
// below walks the reference's own BVH (BVH::build, FEM-AABB/BVH.cu:180) on the
// host with the same stack discipline and the same hex-branch policy, and
// additionally records the element and face ids, which the reference's
// HitRecord does not carry.
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <thread>
#include <atomic>

#include "fem/ModalBasis.cuh"
#include "fem/PrismElement.cuh"
#include "fem/QuadElement.cuh"
#include "fem/TriElement.cuh"
#include "high_order.h"
#include "raytracer.h"
#include "vtu_loader.h"
#include "xml_fld_loader.h"

namespace {

struct RefScene {
  std::vector<zidingyi::HexElementData> hexes;
  std::vector<float> geom, field;
  std::vector<int64_t> goff, foff;
  BVH bvh;
  bool bvh_built = false;
};

void patch_pointers(RefScene& s) {
  for (size_t i = 0; i < s.hexes.size(); ++i) {
    auto& h = s.hexes[i];
    if (s.goff[i] >= 0) {
      const size_t cnt = size_t(h.geomModes.x) * h.geomModes.y * h.geomModes.z;
      h.geomCoefficients[0] = s.geom.data() + s.goff[i];
      h.geomCoefficients[1] = s.geom.data() + s.goff[i] + cnt;
      h.geomCoefficients[2] = s.geom.data() + s.goff[i] + 2 * cnt;
    } else {
      h.geomCoefficients[0] = h.geomCoefficients[1] = h.geomCoefficients[2] = nullptr;
    }
    h.fieldCoefficients = s.foff[i] >= 0 ? s.field.data() + s.foff[i] : nullptr;
  }
}

}  // namespace

extern "C" {

// Scene from flat arrays (same layout as the oracle's scene description).
// Element boxes are computed with the reference's ComputeHexAabb(...,6), as
// its loader does (FEM-AABB/xml_fld_loader.cpp:271-274).
void* ref_scene_create(int n, const uint32_t* gm, const int64_t* goff, const float* geom, int64_t ngeom,
                       const uint32_t* fm, const int64_t* foff, const float* field, int64_t nfield,
                       const float* verts) {
  RefScene* s = new RefScene();
  s->geom.assign(geom, geom + ngeom);
  s->field.assign(field, field + nfield);
  s->goff.assign(goff, goff + n);
  s->foff.assign(foff, foff + n);
  s->hexes.resize(n);
  for (int i = 0; i < n; ++i) {
    zidingyi::HexElementData h{};
    for (int v = 0; v < 8; ++v)
      h.vertices[v] = make_float3(verts[(i * 8 + v) * 3], verts[(i * 8 + v) * 3 + 1], verts[(i * 8 + v) * 3 + 2]);
    h.geomModes = goff[i] >= 0 ? make_uint3(gm[3 * i], gm[3 * i + 1], gm[3 * i + 2]) : make_uint3(0, 0, 0);
    h.fieldModes = make_uint3(fm[3 * i], fm[3 * i + 1], fm[3 * i + 2]);
    s->hexes[i] = h;
  }
  patch_pointers(*s);
  for (auto& h : s->hexes) {
    float3 lo, hi;
    zidingyi::ComputeHexAabb(h, lo, hi, 6);
    h.aabbMin = lo;
    h.aabbMax = hi;
  }
  return s;
}

// Scene through the reference loader (FEM-AABB/xml_fld_loader.cpp:16).
void* ref_scene_load(const char* xml, const char* fld) {
  Scene sc;
  if (!load_xml_fld(xml, fld, sc)) return nullptr;
  RefScene* s = new RefScene();
  s->hexes = sc.hexes;
  s->geom = sc.hex_geom_coefficients;
  s->field = sc.hex_coefficients;
  for (size_t i = 0; i < sc.hexes.size(); ++i) {
    s->goff.push_back(sc.hex_geom_offsets[i]);
    s->foff.push_back(sc.hex_coeff_offsets[i]);
  }
  patch_pointers(*s);
  return s;
}

// Scene through the reference's VTU loader (FEM-AABB/vtu_loader.cpp:156);
// counts3 gets the hexahedra, prisms and quads it added. nullptr when the
// loader reports failure.
void* ref_scene_load_vtu(const char* path, int64_t* counts3) {
  Scene sc;
  const bool ok = load_vtu_file(path, sc);
  counts3[0] = int64_t(sc.hexes.size());
  counts3[1] = int64_t(sc.prisms.size());
  counts3[2] = int64_t(sc.quads.size());
  if (!ok) return nullptr;
  RefScene* s = new RefScene();
  s->hexes = sc.hexes;
  s->geom = sc.hex_geom_coefficients;
  s->field = sc.hex_coefficients;
  for (size_t i = 0; i < sc.hexes.size(); ++i) {
    s->goff.push_back(sc.hex_geom_offsets[i]);
    s->foff.push_back(sc.hex_coeff_offsets[i]);
  }
  patch_pointers(*s);
  return s;
}

// One prism (kind 0), quad (1) or curved triangle (2) built the way
// Scene::add_prism / add_quad / add_curved_tri keep it (FEM-AABB/raytracer.h:
// 167-300): vertices, and modal geometry when gx is given. box6 gets the
// reference's sampled box (ComputePrismAabb / ComputeQuadAabb at 4, and
// ComputeTriAabb at 6 per edge, as raytracer.cu:258-328 calls them); out5 per
// ray the reference's IntersectRayWith* on [seg0, seg1]: (hit, t, r, s, t-coordinate).
int ref_prim_intersect(int kind, const float* verts, const uint32_t* gm3, const float* gx, const float* gy,
                       const float* gz, const float* rays, int64_t n, const double* seg, float* box6,
                       double* out5) {
  float3 lo, hi;
  auto ray_of = [&](int64_t i) {
    zidingyi::Ray r;
    r.origin = make_float3(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]);
    r.direction = make_float3(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
    return r;
  };
  if (kind == 0) {
    zidingyi::PrismElementData e{};
    for (int v = 0; v < 6; ++v) e.vertices[v] = make_float3(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]);
    if (gx) {
      e.geomCoefficients[0] = gx; e.geomCoefficients[1] = gy; e.geomCoefficients[2] = gz;
      e.geomModes = make_uint3(gm3[0], gm3[1], gm3[2]);
    }
    zidingyi::ComputePrismAabb(e, lo, hi, 4);
    for (int64_t i = 0; i < n; ++i) {
      float t; float3 x;
      const bool ok = zidingyi::IntersectRayWithPrism(e, ray_of(i), float(seg[2 * i]), float(seg[2 * i + 1]), t, x);
      double* o = out5 + 5 * i;
      o[0] = ok; o[1] = ok ? t : 0; o[2] = ok ? x.x : 0; o[3] = ok ? x.y : 0; o[4] = ok ? x.z : 0;
    }
  } else if (kind == 1) {
    zidingyi::QuadElementData e{};
    for (int v = 0; v < 4; ++v) e.vertices[v] = make_float3(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]);
    if (gx) {
      e.geomCoefficients[0] = gx; e.geomCoefficients[1] = gy; e.geomCoefficients[2] = gz;
      e.geomModes = make_uint2(gm3[0], gm3[1]);
    }
    zidingyi::ComputeQuadAabb(e, lo, hi, 4);
    for (int64_t i = 0; i < n; ++i) {
      float t; float2 x;
      const bool ok = zidingyi::IntersectRayWithQuad(e, ray_of(i), float(seg[2 * i]), float(seg[2 * i + 1]), t, x);
      double* o = out5 + 5 * i;
      o[0] = ok; o[1] = ok ? t : 0; o[2] = ok ? x.x : 0; o[3] = ok ? x.y : 0; o[4] = 0;
    }
  } else {
    zidingyi::TriElementData e{};
    for (int v = 0; v < 3; ++v) e.vertices[v] = make_float3(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]);
    if (gx) {
      e.geomCoefficients[0] = gx; e.geomCoefficients[1] = gy; e.geomCoefficients[2] = gz;
      e.geomModes = make_uint2(gm3[0], gm3[1]);
    }
    zidingyi::ComputeTriAabb(e, lo, hi, 6);
    for (int64_t i = 0; i < n; ++i) {
      float t; float2 x;
      const bool ok = zidingyi::IntersectRayWithTriangle(e, ray_of(i), float(seg[2 * i]), float(seg[2 * i + 1]), t, x);
      double* o = out5 + 5 * i;
      o[0] = ok; o[1] = ok ? t : 0; o[2] = ok ? x.x : 0; o[3] = ok ? x.y : 0; o[4] = 0;
    }
  }
  box6[0] = lo.x; box6[1] = lo.y; box6[2] = lo.z;
  box6[3] = hi.x; box6[4] = hi.y; box6[5] = hi.z;
  return 0;
}

// The prisms' (n x 6 x 3) and quads' (n x 4 x 3) vertices the reference's
// VTU loader adds; the arrays hold as many as ref_scene_load_vtu counted.
int ref_vtu_prim_verts(const char* path, float* prism_verts, float* quad_verts) {
  Scene sc;
  load_vtu_file(path, sc);
  for (size_t i = 0; i < sc.prisms.size(); ++i)
    for (int v = 0; v < 6; ++v) {
      prism_verts[(6 * i + v) * 3] = sc.prisms[i].vertices[v].x;
      prism_verts[(6 * i + v) * 3 + 1] = sc.prisms[i].vertices[v].y;
      prism_verts[(6 * i + v) * 3 + 2] = sc.prisms[i].vertices[v].z;
    }
  for (size_t i = 0; i < sc.quads.size(); ++i)
    for (int v = 0; v < 4; ++v) {
      quad_verts[(4 * i + v) * 3] = sc.quads[i].vertices[v].x;
      quad_verts[(4 * i + v) * 3 + 1] = sc.quads[i].vertices[v].y;
      quad_verts[(4 * i + v) * 3 + 2] = sc.quads[i].vertices[v].z;
    }
  return 0;
}

void ref_scene_destroy(void* p) { delete static_cast<RefScene*>(p); }

int ref_scene_count(void* p) { return int(static_cast<RefScene*>(p)->hexes.size()); }

// Per element: geom modes(3), field modes(3), geom offset, field offset,
// vertices(24), loader box(6).
int ref_scene_elem(void* p, int i, uint32_t* modes6, int64_t* offs2, float* verts24, float* box6) {
  RefScene* s = static_cast<RefScene*>(p);
  const auto& h = s->hexes[i];
  modes6[0] = h.geomModes.x; modes6[1] = h.geomModes.y; modes6[2] = h.geomModes.z;
  modes6[3] = h.fieldModes.x; modes6[4] = h.fieldModes.y; modes6[5] = h.fieldModes.z;
  offs2[0] = s->goff[i];
  offs2[1] = s->foff[i];
  for (int v = 0; v < 8; ++v) {
    verts24[3 * v] = h.vertices[v].x; verts24[3 * v + 1] = h.vertices[v].y; verts24[3 * v + 2] = h.vertices[v].z;
  }
  box6[0] = h.aabbMin.x; box6[1] = h.aabbMin.y; box6[2] = h.aabbMin.z;
  box6[3] = h.aabbMax.x; box6[4] = h.aabbMax.y; box6[5] = h.aabbMax.z;
  return 0;
}

int64_t ref_scene_geom(void* p, float* out) {
  RefScene* s = static_cast<RefScene*>(p);
  if (out) std::memcpy(out, s->geom.data(), s->geom.size() * sizeof(float));
  return int64_t(s->geom.size());
}

int64_t ref_scene_field(void* p, float* out) {
  RefScene* s = static_cast<RefScene*>(p);
  if (out) std::memcpy(out, s->field.data(), s->field.size() * sizeof(float));
  return int64_t(s->field.size());
}

int ref_basis(unsigned nmodes, float x, float* out) {
  for (unsigned i = 0; i < nmodes; ++i) {
    out[2 * i] = zidingyi::ModifiedA(i, x);
    out[2 * i + 1] = zidingyi::ModifiedAPrime(i, x);
  }
  return 0;
}

int ref_box(void* p, int elem, int samples, float* out6) {
  RefScene* s = static_cast<RefScene*>(p);
  float3 lo, hi;
  zidingyi::ComputeHexAabb(s->hexes[elem], lo, hi, samples);
  out6[0] = lo.x; out6[1] = lo.y; out6[2] = lo.z; out6[3] = hi.x; out6[4] = hi.y; out6[5] = hi.z;
  return 0;
}

int ref_map_point(void* p, int elem, const float* xi, int64_t n, float* out) {
  RefScene* s = static_cast<RefScene*>(p);
  for (int64_t i = 0; i < n; ++i) {
    float3 x = zidingyi::ReferenceToWorldHex(s->hexes[elem], make_float3(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]));
    out[3 * i] = x.x; out[3 * i + 1] = x.y; out[3 * i + 2] = x.z;
  }
  return 0;
}

// 9 Jacobian entries + field value + 3 world-gradient entries per point.
int ref_eval_point(void* p, int elem, const float* xi, int64_t n, float* out) {
  RefScene* s = static_cast<RefScene*>(p);
  const auto& h = s->hexes[elem];
  for (int64_t i = 0; i < n; ++i) {
    const float3 r = make_float3(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]);
    float J[9];
    if (zidingyi::HasHighOrderGeom(h)) zidingyi::JacobianHighOrder(h, r, J);
    else zidingyi::JacobianTrilinear(h, r, J);
    float* o = out + 13 * i;
    for (int k = 0; k < 9; ++k) o[k] = J[k];
    o[9] = h.fieldCoefficients ? zidingyi::EvaluateModalField(h, r) : 0.f;
    float3 g = h.fieldCoefficients ? zidingyi::EvaluateModalGradientWorld(h, r) : make_float3(0, 0, 0);
    o[10] = g.x; o[11] = g.y; o[12] = g.z;
  }
  return 0;
}

int ref_inverse_map(void* p, int elem, const float* x, int64_t n, float* out) {
  RefScene* s = static_cast<RefScene*>(p);
  for (int64_t i = 0; i < n; ++i) {
    float3 r;
    const bool ok = zidingyi::WorldToReferenceNewton(s->hexes[elem], make_float3(x[3 * i], x[3 * i + 1], x[3 * i + 2]), r);
    out[4 * i] = r.x; out[4 * i + 1] = r.y; out[4 * i + 2] = r.z; out[4 * i + 3] = ok ? 1.f : 0.f;
  }
  return 0;
}

int ref_find_iso(void* p, int elem, const float* rays, const float* seg, int64_t n, float iso, float* out) {
  RefScene* s = static_cast<RefScene*>(p);
  for (int64_t i = 0; i < n; ++i) {
    zidingyi::Ray ray;
    ray.origin = make_float3(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]);
    ray.direction = make_float3(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
    float th = 0.f;
    float3 r = make_float3(0, 0, 0), g = make_float3(0, 0, 0);
    const bool ok = zidingyi::FindIsosurfaceOnRayHex(s->hexes[elem], ray, seg[2 * i], seg[2 * i + 1], iso, th, r, g);
    float* o = out + 8 * i;
    o[0] = ok; o[1] = th; o[2] = r.x; o[3] = r.y; o[4] = r.z; o[5] = g.x; o[6] = g.y; o[7] = g.z;
  }
  return 0;
}

int ref_hit_hex(void* p, int elem, const float* rays, const float* seg, int64_t n, float* out) {
  RefScene* s = static_cast<RefScene*>(p);
  for (int64_t i = 0; i < n; ++i) {
    zidingyi::Ray ray;
    ray.origin = make_float3(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]);
    ray.direction = make_float3(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
    float th = 0.f;
    float3 r = make_float3(0, 0, 0);
    int face = -1;
    const bool ok = IntersectRayWithHex(s->hexes[elem], ray, seg[2 * i], seg[2 * i + 1], th, r, face);
    float* o = out + 6 * i;
    o[0] = ok; o[1] = th; o[2] = r.x; o[3] = r.y; o[4] = r.z; o[5] = float(face);
  }
  return 0;
}

// Host walk of the reference BVH with bvh_intersect_device's stack order and
// hex policy (FEM-AABB/raytracer.cu:111-358). out per ray (12 floats):
// kind (0 miss, 1 face, 2 iso), elem, face, t, xi(3), normal(3), material, pad.
// order (optional, n x order_cap): elements visited (box test passed), in
// visit order, -1 padded; order_n[i] = how many (may exceed order_cap).
// iso_mode: 0 = the renderer's rule (isovalue 0 turns the isosurface off,
// raytracer.cu:207); 1 = FindIsosurfaceOnRayHex is called for every
// isovalue, 0 included (how an isovalue of 0 is compared at all).
int ref_trace_order_iso(void* p, const float* rays, int64_t n, float iso, int iso_mode, float* out, int32_t* order,
                        int order_cap, int32_t* order_n);
int ref_trace_order(void* p, const float* rays, int64_t n, float iso, float* out, int32_t* order, int order_cap,
                    int32_t* order_n) {
  return ref_trace_order_iso(p, rays, n, iso, 0, out, order, order_cap, order_n);
}
int ref_trace(void* p, const float* rays, int64_t n, float iso, float* out) {
  return ref_trace_order_iso(p, rays, n, iso, 0, out, nullptr, 0, nullptr);
}
int ref_trace_order_iso(void* p, const float* rays, int64_t n, float iso, int iso_mode, float* out, int32_t* order,
                        int order_cap, int32_t* order_n) {
  RefScene* s = static_cast<RefScene*>(p);
  if (!s->bvh_built) {
    std::vector<Sphere> sp;
    std::vector<Triangle> tr;
    std::vector<zidingyi::PrismElementData> pr;
    std::vector<zidingyi::QuadElementData> qu;
    std::vector<zidingyi::TriElementData> ct;
    s->bvh.build(sp, tr, s->hexes, pr, qu, ct);
    s->bvh_built = true;
  }
  const auto& nodes = s->bvh.nodes;
  const auto& prims = s->bvh.primitive_indices;
  // rays are independent: the reference's element routines keep no state,
  // so the host walk runs on every hardware thread (each ray writes its own
  // output slots)
  std::atomic<int64_t> next_ray{0};
  auto walk = [&] {
  for (;;) {
    const int64_t ri = next_ray.fetch_add(1);
    if (ri >= n) break;
    ::Ray ray(make_float3(rays[6 * ri], rays[6 * ri + 1], rays[6 * ri + 2]),
              make_float3(rays[6 * ri + 3], rays[6 * ri + 4], rays[6 * ri + 5]));
    float rec_t = FLT_MAX;
    int kind = 0, hit_elem = -1, hit_face = -1, mat = -1;
    float3 hit_xi = make_float3(0, 0, 0), hit_n = make_float3(0, 0, 0);
    int todo[64];
    int top = 0;
    int nvis = 0;
    if (order)
      for (int k = 0; k < order_cap; ++k) order[ri * order_cap + k] = -1;
    if (!nodes.empty()) todo[top++] = 0;
    while (top > 0) {
      const BVHNode& node = nodes[todo[--top]];
      float tb0, tb1;
      if (!node.bounds.intersect(ray, tb0, tb1) || tb0 >= rec_t) continue;
      if (node.is_leaf) {
        for (int i = 0; i < node.right_child_or_count; ++i) {
          const int enc = prims[node.left_child_or_primitive + i];
          if (DecodePrimitiveType(enc) != PrimitiveType::Hex) continue;
          const int ei = DecodePrimitiveIndex(enc);
          const zidingyi::HexElementData& elem = s->hexes[ei];
          float3 lo, hi;
          zidingyi::ComputeHexAabb(elem, lo, hi, 4);
          float te, tx;
          zidingyi::Ray hr = ToHighOrderRay(ray);
          if (!RayAabbIntersectHO(hr, lo, hi, 0.001f, rec_t, te, tx)) continue;
          if (order && nvis < order_cap) order[ri * order_cap + nvis] = ei;
          ++nvis;
          float th;
          float3 rst, g;
          const bool iso_ok = (iso_mode == 1 || iso != 0.0f) && elem.fieldCoefficients != nullptr && elem.fieldModes.x > 0 &&
                              elem.fieldModes.y > 0 && elem.fieldModes.z > 0;
          if (iso_ok && zidingyi::FindIsosurfaceOnRayHex(elem, hr, te, tx, iso, th, rst, g)) {
            if (th > 0.001f && th < rec_t) {
              rec_t = th;
              float3 nn = normalize(g);
              if (dot(nn, ray.direction) > 0.0f) nn = -nn;
              kind = 2; hit_elem = ei; hit_face = -1; hit_xi = rst; hit_n = nn; mat = 0;
            }
          } else {
            int fidx = -1;
            if (IntersectRayWithHex(elem, hr, 0.001f, rec_t, th, rst, fidx)) {
              if (th > 0.001f && th < rec_t) {
                rec_t = th;
                float J[9];
                if (zidingyi::HasHighOrderGeom(elem)) zidingyi::JacobianHighOrder(elem, rst, J);
                else zidingyi::JacobianTrilinear(elem, rst, J);
                const float3 dr = make_float3(J[0], J[3], J[6]), ds = make_float3(J[1], J[4], J[7]),
                             dt = make_float3(J[2], J[5], J[8]);
                float3 nn;
                if (fabsf(rst.x) > 0.9f) nn = cross(ds, dt);
                else if (fabsf(rst.y) > 0.9f) nn = cross(dr, dt);
                else nn = cross(dr, ds);
                nn = normalize(nn);
                if (dot(nn, ray.direction) > 0.0f) nn = -nn;
                kind = 1; hit_elem = ei; hit_face = fidx; hit_xi = rst; hit_n = nn; mat = (fidx == 0) ? 1 : 0;
              }
            }
          }
        }
      } else if (top < 62) {
        todo[top++] = node.left_child_or_primitive;
        todo[top++] = node.right_child_or_count;
      }
    }
    if (order_n) order_n[ri] = nvis;
    float* o = out + 12 * ri;
    o[0] = float(kind); o[1] = float(hit_elem); o[2] = float(hit_face); o[3] = kind ? rec_t : FLT_MAX;
    o[4] = hit_xi.x; o[5] = hit_xi.y; o[6] = hit_xi.z;
    o[7] = hit_n.x; o[8] = hit_n.y; o[9] = hit_n.z;
    o[10] = float(mat); o[11] = 0.f;
  }
  };
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  std::vector<std::thread> pool;
  for (unsigned k = 1; k < nt; ++k) pool.emplace_back(walk);
  walk();
  for (auto& th : pool) th.join();
  return 0;
}

}  // extern "C"
