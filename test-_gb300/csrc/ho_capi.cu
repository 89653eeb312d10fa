// C ABI of the renderer (declared in include/horender.h).
//
// A context owns one CUDA stream and the device copy of one scene. The CUDA
// context is touched lazily (first build / render), so scene assembly and
// the host-side loader work without a GPU. Every call returns an HO_* status
// and leaves its message in ho_last_error(); nothing throws across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "ho_host.h"
#include "ho_learn.h"
#include "ho_mlp.h"

using ho::HostScene;

namespace {

int fail(ho_context* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(ho_context* c, int e, const char* what) {
  return fail(c, HO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(static_cast<cudaError_t>(e)));
}

#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t e__ = (call);                            \
    if (e__ != cudaSuccess) return cuda_fail(c, int(e__), what); \
  } while (0)

int ensure_device(ho_context* c) {
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (!c->stream) CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  if (!c->d_stats) CK(cudaMalloc(&c->d_stats, sizeof(ho::DevStats)), "cudaMalloc(stats)");
  return HO_OK;
}

void free_scene(ho_context* c) {
  cudaFree(c->d_rec);
  cudaFree(c->d_box);
  cudaFree(c->d_hull);
  cudaFree(c->d_fbox);
  cudaFree(c->d_flags);
  cudaFree(c->d_own);
  cudaFree(c->d_nodes);
  cudaFree(c->d_desc);
  cudaFree(c->d_crec);
  cudaFree(c->d_coff);
  cudaFree(c->d_cord);
  c->d_crec = nullptr;
  c->d_coff = nullptr;
  c->d_cord = nullptr;
  c->orders = 0;
  c->d_desc = nullptr;
  c->d_rec = c->d_box = c->d_hull = c->d_fbox = nullptr;
  c->d_flags = nullptr;
  c->d_own = nullptr;
  c->d_nodes = nullptr;
  c->n_elem = 0;
  ho::prims_free(c);
  c->built = false;
  c->device_bytes = 0;
}

template <class T>
int ensure_buf(ho_context* c, T*& p, size_t& cap, size_t count, const char* what) {
  if (count <= cap && p) return HO_OK;
  cudaFree(p);
  p = nullptr;
  cap = 0;
  CK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), what);
  cap = count;
  return HO_OK;
}

// Pinhole camera basis (FEM-AABB/raytracer.h:31-48, aperture 0).
void camera_basis(const ho_camera& cam, int W, int H, ho::TraceArgs& a) {
  auto sub = [](const float* x, const float* y, float* o) {
    for (int i = 0; i < 3; ++i) o[i] = x[i] - y[i];
  };
  auto len = [](const float* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
  auto cross = [](const float* x, const float* y, float* o) {
    o[0] = x[1] * y[2] - x[2] * y[1];
    o[1] = x[2] * y[0] - x[0] * y[2];
    o[2] = x[0] * y[1] - x[1] * y[0];
  };
  const float theta = cam.vfov_deg * 3.14159265f / 180.0f;
  const float h = std::tan(theta / 2.0f);
  const float vh = 2.0f * h, vw = (static_cast<float>(W) / static_cast<float>(H)) * vh;
  float w[3], u[3], v[3];
  sub(cam.lookfrom, cam.lookat, w);
  float focus = cam.focus_dist > 0.f ? cam.focus_dist : len(w);
  const float lw = len(w);
  for (float& x : w) x = x * (1.0f / lw);
  cross(cam.vup, w, u);
  const float lu = len(u);
  for (float& x : u) x = x * (1.0f / lu);
  cross(w, u, v);
  for (int i = 0; i < 3; ++i) {
    a.origin[i] = cam.lookfrom[i];
    a.horiz[i] = focus * vw * u[i];
    a.vert[i] = focus * vh * v[i];
    a.llc[i] = cam.lookfrom[i] - a.horiz[i] / 2.0f - a.vert[i] / 2.0f - focus * w[i];
  }
  a.width = W;
  a.height = H;
}

// End of a *_device call on stream s: later stats reads wait for it. A
// stream the caller is capturing gets no event (nothing has run yet).
int mark_call_done(ho_context* c, cudaStream_t s) {
  c->call_done_pending = false;
  if (s == c->stream) return HO_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(s, &cs), "cudaStreamIsCapturing");
  if (cs != cudaStreamCaptureStatusNone) return HO_OK;
  if (!c->call_done) CK(cudaEventCreateWithFlags(&c->call_done, cudaEventDisableTiming), "cudaEventCreate");
  CK(cudaEventRecord(c->call_done, s), "cudaEventRecord");
  c->call_done_pending = true;
  return HO_OK;
}

int read_stats(ho_context* c) {
  ho::DevStats ds;
  if (c->call_done_pending) CK(cudaStreamWaitEvent(c->stream, c->call_done, 0), "cudaStreamWaitEvent");
  CK(cudaMemcpyAsync(&ds, c->d_stats, sizeof(ds), cudaMemcpyDeviceToHost, c->stream), "read stats");
  CK(cudaStreamSynchronize(c->stream), "sync");
  ho_stats& s = c->last;
  s.rays = ds.c[ho::ST_RAYS];
  s.candidates = ds.c[ho::ST_CAND];
  s.geom_evals = ds.c[ho::ST_GEOM];
  s.map_evals = ds.c[ho::ST_MAP];
  s.field_evals = ds.c[ho::ST_FIELD];
  s.newton_iters = ds.c[ho::ST_NEWTON];
  s.face_iters = ds.c[ho::ST_FACE];
  s.faces_culled = ds.c[ho::ST_CULLED];
  s.node_visits = ds.c[ho::ST_NODES];
  s.mlp_accepted = ds.c[ho::ST_ACCEPT];
  s.mlp_rejected = ds.c[ho::ST_REJECT];
  s.restarts = ds.c[ho::ST_RESTART];
  for (int k = 0; k < 4; ++k) s.phase_cycles[k] = ds.c[ho::ST_CYC_TRAV + k];
  s.max_modes = c->N;
  s.status = ds.status;
  s.rounds = ds.c[ho::ST_ROUNDS];
  s.round_pairs = ds.c[ho::ST_PAIRS];
  s.graph = c->last_graph ? 1u : 0u;
  s.fp64_checked = ds.c[ho::ST_CHECKED];
  s.fp64_failed = ds.c[ho::ST_CHECK_FAIL];
  s.fp64_failed_after_fallback = ds.c[ho::ST_CHECK_FINAL];
  s.round_flops = ds.c[ho::ST_FLOPS];
  s.solve_steps = ds.c[ho::ST_STEPS];
  s.lane_steps = ds.c[ho::ST_LANES];
  s.tail_rays = ds.c[ho::ST_TAIL];
  s.prim_candidates = ds.c[ho::ST_PRIM_CAND];
  s.prim_iters = ds.c[ho::ST_PRIM_ITERS];
  s.prim_flops = ds.c[ho::ST_PRIM_FLOPS];
  s.prim_node_visits = ds.c[ho::ST_PRIM_NODES];
  s.fp64_polished = ds.c[ho::ST_POLISHED];
  s.fp64_ties = ds.c[ho::ST_TIES];
  s.fp64_ties_swapped = ds.c[ho::ST_TIES_SWAPPED];
  s.grazing_hits = ds.c[ho::ST_GRAZING];
  s.prim_kernel_ns = 0;
  if (c->prim_timed) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->prim_events[0], c->prim_events[1]) != cudaSuccess) {
      cudaGetLastError();
      return fail(c, HO_ERR_CUDA, "primitive timing events could not be read");
    }
    s.prim_kernel_ns = static_cast<uint64_t>(static_cast<double>(ms) * 1e6 + 0.5);
  }
  s.kernel_launches = static_cast<uint64_t>(c->launches);
  s.round_kernel_ns = 0;
  s.round_launches = 0;
  for (int k = 0; k + 1 < c->round_events_used; k += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->round_events[k], c->round_events[k + 1]) != cudaSuccess) {
      cudaGetLastError();
      return fail(c, HO_ERR_CUDA, "round timing events could not be read");
    }
    s.round_kernel_ns += static_cast<uint64_t>(static_cast<double>(ms) * 1e6 + 0.5);
    s.round_launches += static_cast<uint64_t>(__builtin_popcount(c->orders));
  }
  if (ds.status != 0)
    return fail(c, HO_ERR_DEVICE, "kernel reported status " + std::to_string(ds.status) +
                                      (ds.status & ho::kStatusStackOverflow ? " (traversal stack overflow)" : "") +
                                      (ds.status & ho::kStatusRoundGuard ? " (intersection round did not finish)" : ""));
  return HO_OK;
}

int check_iso(ho_context* c, const float* iso, int n_iso) {
  if (n_iso < 1 || n_iso > 8) return fail(c, HO_ERR_RANGE, "n_iso must be in [1, 8]");
  if (!iso) return fail(c, HO_ERR_ARG, "isovalues is NULL");
  return HO_OK;
}

}  // namespace

extern "C" {

int ho_create(int device, ho_context** out) {
  if (!out) return HO_ERR_ARG;
  *out = nullptr;
  if (device < 0) return HO_ERR_ARG;
  ho_context* c = new (std::nothrow) ho_context();
  if (!c) return HO_ERR_NOMEM;
  c->device = device;
  *out = c;
  return HO_OK;
}

void ho_destroy(ho_context* c) {
  if (!c) return;
  if (c->stream) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_scene(c);
    cudaFree(c->d_stats);
    cudaFree(c->d_hits);
    cudaFree(c->d_phits);
    if (c->prim_events[0]) cudaEventDestroy(c->prim_events[0]);
    if (c->prim_events[1]) cudaEventDestroy(c->prim_events[1]);
    if (c->call_done) cudaEventDestroy(c->call_done);
    cudaFree(c->d_rgb);
    cudaFree(c->d_rays);
    cudaFree(c->d_views);
    cudaFree(c->d_work);
    cudaFree(c->d_kbuf);
    cudaFree(c->d_kovf);
    cudaFree(c->d_qctr);
    cudaFree(c->rounds.state);
    cudaFree(c->rounds.pairs);
    cudaFree(c->rounds.pelem);
    cudaFree(c->rounds.prank);
    cudaFree(c->rounds.batches);
    cudaFree(c->rounds.ecount);
    cudaFree(c->rounds.eoff);
    cudaFree(c->rounds.tile_sums);
    cudaFree(c->rounds.ctr);
    cudaFree(c->rounds.fail);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    for (cudaEvent_t ev : c->round_events) cudaEventDestroy(ev);
    cudaFree(c->d_pred);
    cudaFree(c->d_cand);
    c->mlp.release();
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    cudaStreamDestroy(c->stream);
  }
  delete c;
}

const char* ho_last_error(const ho_context* c) { return c ? c->err.c_str() : "null context"; }

// Every value finite (a NaN or infinite coordinate or coefficient would reach
// the solvers as a NaN iterate; it is refused at the door instead).
static bool all_finite(const float* v, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

int ho_add_hexes(ho_context* c, int64_t n, const float* corners, const uint32_t* gm, const float* geom,
                 int64_t geom_len, const int64_t* goff, const uint32_t* fm, const float* field, int64_t field_len,
                 const int64_t* foff) {
  if (!c) return HO_ERR_ARG;
  if (n < 0) return fail(c, HO_ERR_ARG, "n must be >= 0");
  if (n > 0 && (!corners || !gm || !goff || !fm || !foff)) return fail(c, HO_ERR_ARG, "null array");
  HostScene& hs = c->hs;
  // validate first, so a failed call leaves the scene unchanged
  for (int64_t i = 0; i < n; ++i) {
    if (goff[i] >= 0) {
      int64_t cnt = 1;
      for (int a = 0; a < 3; ++a) {
        if (gm[3 * i + a] < ho::kMinModes || gm[3 * i + a] > ho::kMaxModes)
          return fail(c, HO_ERR_RANGE, "element " + std::to_string(i) + ": geometry modes must be in [2, 9]");
        cnt *= gm[3 * i + a];
      }
      if (!geom || goff[i] + 3 * cnt > geom_len)
        return fail(c, HO_ERR_ARG, "element " + std::to_string(i) + ": geometry coefficients out of range");
      if (!all_finite(geom + goff[i], 3 * cnt))
        return fail(c, HO_ERR_ARG, "element " + std::to_string(i) + ": non-finite geometry coefficient");
    }
    if (!all_finite(corners + 24 * i, 24))
      return fail(c, HO_ERR_ARG, "element " + std::to_string(i) + ": non-finite corner");
    if (foff[i] >= 0) {
      int64_t cnt = 1;
      for (int a = 0; a < 3; ++a) {
        if (fm[3 * i + a] < 1 || fm[3 * i + a] > ho::kMaxModes)
          return fail(c, HO_ERR_RANGE, "element " + std::to_string(i) + ": field modes must be in [1, 9]");
        cnt *= fm[3 * i + a];
      }
      if (!field || foff[i] + cnt > field_len)
        return fail(c, HO_ERR_ARG, "element " + std::to_string(i) + ": field coefficients out of range");
      if (!all_finite(field + foff[i], cnt))
        return fail(c, HO_ERR_ARG, "element " + std::to_string(i) + ": non-finite field coefficient");
    }
  }
  for (int64_t i = 0; i < n; ++i) {
    hs.corners.insert(hs.corners.end(), corners + 24 * i, corners + 24 * i + 24);
    if (goff[i] >= 0) {
      const int64_t cnt = static_cast<int64_t>(gm[3 * i]) * gm[3 * i + 1] * gm[3 * i + 2];
      hs.goff.push_back(static_cast<int64_t>(hs.geom.size()));
      hs.geom.insert(hs.geom.end(), geom + goff[i], geom + goff[i] + 3 * cnt);
      for (int a = 0; a < 3; ++a) hs.gmodes.push_back(gm[3 * i + a]);
    } else {
      hs.goff.push_back(-1);
      for (int a = 0; a < 3; ++a) hs.gmodes.push_back(0);
    }
    if (foff[i] >= 0) {
      const int64_t cnt = static_cast<int64_t>(fm[3 * i]) * fm[3 * i + 1] * fm[3 * i + 2];
      hs.foff.push_back(static_cast<int64_t>(hs.field.size()));
      hs.field.insert(hs.field.end(), field + foff[i], field + foff[i] + cnt);
    } else {
      hs.foff.push_back(-1);
    }
    for (int a = 0; a < 3; ++a) hs.fmodes.push_back(fm[3 * i + a]);
  }
  c->built = false;
  return HO_OK;
}

namespace {

// Coefficients in one component block of a primitive kind (m: its modes).
int64_t prim_block_len(int kind, const uint32_t m[3]) {
  if (kind == 1) return static_cast<int64_t>(m[0]) * m[1];
  const int64_t top = kind == 0 ? m[2] : m[1];
  int64_t n = 0;
  for (int64_t i = 0; i < m[0]; ++i) n += std::max<int64_t>(top - i, 0);
  return kind == 0 ? n * m[1] : n;
}

// ho_add_prisms / quads / tris: dims modes per primitive (3 or 2), nv vertices.
int add_prims(ho_context* c, int kind, int nv, int dims, int64_t n, const float* verts, const uint32_t* gm,
              const float* geom, int64_t geom_len, const int64_t* goff, const uint32_t* fm, const float* field,
              int64_t field_len, const int64_t* foff) {
  if (!c) return HO_ERR_ARG;
  if (n < 0) return fail(c, HO_ERR_ARG, "n must be >= 0");
  if (n > 0 && (!verts || !gm || !goff || !fm || !foff)) return fail(c, HO_ERR_ARG, "null array");
  ho::HostPrims& hp = c->hs.prims;
  if (hp.size() + n > (int64_t(1) << 30)) return fail(c, HO_ERR_RANGE, "at most 2^30 primitives");
  auto modes = [&](const uint32_t* src, int64_t i, uint32_t out[3]) {
    out[0] = src[dims * i];
    out[1] = src[dims * i + 1];
    out[2] = dims == 3 ? src[dims * i + 2] : 0u;
  };
  for (int64_t i = 0; i < n; ++i) {
    uint32_t m[3];
    if (goff[i] >= 0) {
      modes(gm, i, m);
      for (int a = 0; a < dims; ++a)
        if (m[a] < 1 || m[a] > ho::kMaxModes)
          return fail(c, HO_ERR_RANGE, "primitive " + std::to_string(i) + ": geometry modes must be in [1, 9]");
      if (!geom || goff[i] + 3 * prim_block_len(kind, m) > geom_len)
        return fail(c, HO_ERR_ARG, "primitive " + std::to_string(i) + ": geometry coefficients out of range");
      if (!all_finite(geom + goff[i], 3 * prim_block_len(kind, m)))
        return fail(c, HO_ERR_ARG, "primitive " + std::to_string(i) + ": non-finite geometry coefficient");
    }
    if (!all_finite(verts + static_cast<int64_t>(nv) * 3 * i, nv * 3))
      return fail(c, HO_ERR_ARG, "primitive " + std::to_string(i) + ": non-finite vertex");
    if (foff[i] >= 0) {
      modes(fm, i, m);
      for (int a = 0; a < dims; ++a)
        if (m[a] < 1 || m[a] > ho::kMaxModes)
          return fail(c, HO_ERR_RANGE, "primitive " + std::to_string(i) + ": field modes must be in [1, 9]");
      if (!field || foff[i] + prim_block_len(kind, m) > field_len)
        return fail(c, HO_ERR_ARG, "primitive " + std::to_string(i) + ": field coefficients out of range");
      if (!all_finite(field + foff[i], prim_block_len(kind, m)))
        return fail(c, HO_ERR_ARG, "primitive " + std::to_string(i) + ": non-finite field coefficient");
    }
  }
  for (int64_t i = 0; i < n; ++i) {
    hp.kind.push_back(kind);
    const size_t at = hp.verts.size();
    hp.verts.resize(at + 18, 0.0f);
    std::copy(verts + 3 * nv * i, verts + 3 * nv * (i + 1), hp.verts.begin() + at);
    uint32_t m[3];
    if (goff[i] >= 0) {
      modes(gm, i, m);
      const int64_t cnt = 3 * prim_block_len(kind, m);
      hp.goff.push_back(static_cast<int64_t>(hp.geom.size()));
      hp.geom.insert(hp.geom.end(), geom + goff[i], geom + goff[i] + cnt);
    } else {
      m[0] = m[1] = m[2] = 0;
      hp.goff.push_back(-1);
    }
    hp.gmodes.insert(hp.gmodes.end(), m, m + 3);
    modes(fm, i, m);
    if (foff[i] >= 0) {
      const int64_t cnt = prim_block_len(kind, m);
      hp.foff.push_back(static_cast<int64_t>(hp.field.size()));
      hp.field.insert(hp.field.end(), field + foff[i], field + foff[i] + cnt);
    } else {
      hp.foff.push_back(-1);
    }
    hp.fmodes.insert(hp.fmodes.end(), m, m + 3);
  }
  c->built = false;
  return HO_OK;
}

}  // namespace

int ho_add_prisms(ho_context* c, int64_t n, const float* verts, const uint32_t* gm, const float* geom, int64_t geom_len,
                  const int64_t* goff, const uint32_t* fm, const float* field, int64_t field_len, const int64_t* foff) {
  return add_prims(c, 0, 6, 3, n, verts, gm, geom, geom_len, goff, fm, field, field_len, foff);
}

int ho_add_quads(ho_context* c, int64_t n, const float* verts, const uint32_t* gm, const float* geom, int64_t geom_len,
                 const int64_t* goff, const uint32_t* fm, const float* field, int64_t field_len, const int64_t* foff) {
  return add_prims(c, 1, 4, 2, n, verts, gm, geom, geom_len, goff, fm, field, field_len, foff);
}

int ho_add_tris(ho_context* c, int64_t n, const float* verts, const uint32_t* gm, const float* geom, int64_t geom_len,
                const int64_t* goff, const uint32_t* fm, const float* field, int64_t field_len, const int64_t* foff) {
  return add_prims(c, 2, 3, 2, n, verts, gm, geom, geom_len, goff, fm, field, field_len, foff);
}

int ho_get_prims(ho_context* c, int64_t* n, int32_t* kind, float* verts, uint32_t* gm, float* geom, int64_t* geom_len,
                 int64_t* goff, uint32_t* fm, float* field, int64_t* field_len, int64_t* foff) {
  if (!c) return HO_ERR_ARG;
  const ho::HostPrims& hp = c->hs.prims;
  if (n) *n = hp.size();
  if (geom_len) *geom_len = static_cast<int64_t>(hp.geom.size());
  if (field_len) *field_len = static_cast<int64_t>(hp.field.size());
  if (geom) std::memcpy(geom, hp.geom.data(), hp.geom.size() * sizeof(float));
  if (field) std::memcpy(field, hp.field.data(), hp.field.size() * sizeof(float));
  int64_t j = 0;
  for (int k = 0; k < 3; ++k)
    for (int64_t i = 0; i < hp.size(); ++i) {
      if (hp.kind[i] != k) continue;
      if (kind) kind[j] = k;
      if (verts) std::memcpy(verts + 18 * j, hp.verts.data() + 18 * i, 18 * sizeof(float));
      if (gm) std::memcpy(gm + 3 * j, hp.gmodes.data() + 3 * i, 3 * sizeof(uint32_t));
      if (fm) std::memcpy(fm + 3 * j, hp.fmodes.data() + 3 * i, 3 * sizeof(uint32_t));
      if (goff) goff[j] = hp.goff[i];
      if (foff) foff[j] = hp.foff[i];
      ++j;
    }
  return HO_OK;
}

int ho_get_prim_boxes(ho_context* c, float* out) {
  if (!c || !out) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (c->n_prims == 0) return HO_OK;
  CK(cudaMemcpyAsync(out, c->d_pbox, c->n_prims * 6 * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "read boxes");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return HO_OK;
}

int ho_generate_synthetic(ho_context* c, const ho_synth_params* p) {
  if (!c) return HO_ERR_ARG;
  if (!p) return fail(c, HO_ERR_ARG, "params is NULL");
  std::string err;
  const int rc = ho::generate_synthetic(*p, c->hs, err);
  if (rc != HO_OK) return fail(c, rc, err);
  c->built = false;
  return HO_OK;
}

int ho_load_xml_fld(ho_context* c, const char* xml, const char* fld) {
  if (!c) return HO_ERR_ARG;
  if (!xml || !fld) return fail(c, HO_ERR_ARG, "path is NULL");
  std::string err;
  bool on_gpu = c->gpu_fit == 1;
  if (c->gpu_fit < 0) {
    int n_dev = 0;
    on_gpu = cudaGetDeviceCount(&n_dev) == cudaSuccess && c->device < n_dev;
    cudaGetLastError();
  }
  std::unique_ptr<ho::ModalFitter> fitter = on_gpu ? ho::make_gpu_fitter(c->device) : ho::make_host_fitter();
  const int rc = ho::load_xml_fld(xml, fld, c->hs, err, fitter.get());
  c->last_fit_gpu = on_gpu;
  if (rc != HO_OK) return fail(c, rc, err);
  c->built = false;
  return HO_OK;
}

int ho_load_vtu(ho_context* c, const char* path) {
  if (!c) return HO_ERR_ARG;
  if (!path) return fail(c, HO_ERR_ARG, "path is NULL");
  std::string err;
  const int rc = ho::load_vtu(path, c->hs, err);
  if (rc != HO_OK) return fail(c, rc, err);
  c->built = false;
  return HO_OK;
}

int ho_get_scene(ho_context* c, int64_t* n, float* corners, uint32_t* gm, float* geom, int64_t* geom_len,
                 int64_t* goff, uint32_t* fm, float* field, int64_t* field_len, int64_t* foff) {
  if (!c) return HO_ERR_ARG;
  const HostScene& hs = c->hs;
  if (n) *n = hs.size();
  if (geom_len) *geom_len = static_cast<int64_t>(hs.geom.size());
  if (field_len) *field_len = static_cast<int64_t>(hs.field.size());
  if (corners) std::memcpy(corners, hs.corners.data(), hs.corners.size() * sizeof(float));
  if (gm) std::memcpy(gm, hs.gmodes.data(), hs.gmodes.size() * sizeof(uint32_t));
  if (geom) std::memcpy(geom, hs.geom.data(), hs.geom.size() * sizeof(float));
  if (goff) std::memcpy(goff, hs.goff.data(), hs.goff.size() * sizeof(int64_t));
  if (fm) std::memcpy(fm, hs.fmodes.data(), hs.fmodes.size() * sizeof(uint32_t));
  if (field) std::memcpy(field, hs.field.data(), hs.field.size() * sizeof(float));
  if (foff) std::memcpy(foff, hs.foff.data(), hs.foff.size() * sizeof(int64_t));
  return HO_OK;
}

int ho_build_bvh(ho_context* c) {
  if (!c) return HO_ERR_ARG;
  const HostScene& hs = c->hs;
  if (hs.size() == 0 && hs.prims.size() == 0) return fail(c, HO_ERR_STATE, "scene is empty");
  if (hs.size() > (int64_t(1) << 30)) return fail(c, HO_ERR_RANGE, "at most 2^30 elements");
  int rc = ensure_device(c);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream), "sync");
  free_scene(c);
  rc = ho::prims_build(c);
  if (rc) return cuda_fail(c, rc, "primitive setup");
  if (c->pbvh_depth + 2 > 64) return fail(c, HO_ERR_RANGE, "primitive BVH deeper than the traversal stack");
  if (hs.size() == 0) {  // primitives only
    c->N = 0;
    c->n_elem = 0;
    CK(cudaStreamSynchronize(c->stream), "sync");
    c->built = true;
    return HO_OK;
  }
  const int N = ho::scene_max_modes(hs);
  if (N > ho::kMaxModes) return fail(c, HO_ERR_RANGE, "modes per direction must be <= 9");
  c->N = N;
  c->n_elem = hs.size();
  std::vector<float> rec;
  std::vector<uint32_t> flags;
  std::vector<int32_t> own;
  ho::pack_records(hs, N, rec, flags, own);
  const int64_t ne = c->n_elem;
  CK(cudaMalloc(&c->d_rec, rec.size() * sizeof(float)), "cudaMalloc(records)");
  CK(cudaMalloc(&c->d_flags, ne * sizeof(uint32_t)), "cudaMalloc(flags)");
  CK(cudaMalloc(&c->d_own, ne * sizeof(int32_t)), "cudaMalloc(own)");
  CK(cudaMalloc(&c->d_box, ne * 6 * sizeof(float)), "cudaMalloc(box)");
  CK(cudaMalloc(&c->d_hull, ne * 6 * sizeof(float)), "cudaMalloc(hull)");
  CK(cudaMalloc(&c->d_fbox, ne * ho::kFaceBoxFloats * sizeof(float)), "cudaMalloc(face boxes)");
  CK(cudaMemcpyAsync(c->d_rec, rec.data(), rec.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream), "upload");
  CK(cudaMemcpyAsync(c->d_flags, flags.data(), ne * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream), "upload");
  CK(cudaMemcpyAsync(c->d_own, own.data(), ne * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream), "upload");
  {
    // per-element orders; a mixed-order scene also gets compact records at
    // each element's own order for the round kernels
    std::vector<uint8_t> ord(ne);
    for (int64_t e = 0; e < ne; ++e) {
      ord[e] = static_cast<uint8_t>(ho::element_order(hs, e));
      c->orders |= 1u << ord[e];
    }
    CK(cudaMalloc(&c->d_cord, ne * sizeof(uint8_t)), "cudaMalloc(orders)");
    CK(cudaMemcpyAsync(c->d_cord, ord.data(), ne, cudaMemcpyHostToDevice, c->stream), "upload");
    if (c->orders != (1u << N)) {
      std::vector<float> crec;
      std::vector<int64_t> coff;
      ho::pack_compact(hs, crec, coff, ord);
      CK(cudaMalloc(&c->d_crec, crec.size() * sizeof(float)), "cudaMalloc(compact records)");
      CK(cudaMalloc(&c->d_coff, ne * sizeof(int64_t)), "cudaMalloc(record offsets)");
      CK(cudaMemcpyAsync(c->d_crec, crec.data(), crec.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream),
         "upload");
      CK(cudaMemcpyAsync(c->d_coff, coff.data(), ne * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream), "upload");
      CK(cudaStreamSynchronize(c->stream), "sync");
      c->device_bytes += static_cast<int64_t>(crec.size() * sizeof(float)) + ne * 8;
    }
  }
  rc = ho::launch_setup(c);
  if (rc) return cuda_fail(c, rc, "setup kernel");
  rc = ho::build_lbvh(c);
  if (rc) return cuda_fail(c, rc, "LBVH build");
  CK(cudaMalloc(&c->d_desc, ne * ho::kDescFloats * sizeof(float)), "cudaMalloc(descriptors)");
  rc = ho::launch_desc(c->N, c->d_rec, ne, c->d_desc, c->stream);
  if (rc) return cuda_fail(c, rc, "descriptor kernel");
  if (c->bvh_depth + 2 > 64) return fail(c, HO_ERR_RANGE, "BVH deeper than the traversal stack");
  CK(cudaStreamSynchronize(c->stream), "sync");
  c->device_bytes += static_cast<int64_t>(rec.size() * sizeof(float)) + ne * (4 + 4 + 1 + 24 + 24 + 144) +
                     c->n_nodes * static_cast<int64_t>(sizeof(ho::BNode));
  c->built = true;
  return HO_OK;
}

int ho_scene_info_get(ho_context* c, ho_scene_info* out) {
  if (!c || !out) return HO_ERR_ARG;
  out->n_elem = c->hs.size();
  out->n_nodes = c->built ? c->n_nodes : 0;
  out->max_modes = c->built ? c->N : ho::scene_max_modes(c->hs);
  out->bvh_depth = c->built ? c->bvh_depth : 0;
  out->device_bytes = c->built ? c->device_bytes : 0;
  for (int i = 0; i < 6; ++i) out->bounds[i] = c->bounds[i];
  int64_t cnt[3] = {0, 0, 0};
  for (int32_t k : c->hs.prims.kind) ++cnt[k];
  out->n_prisms = cnt[0];
  out->n_quads = cnt[1];
  out->n_tris = cnt[2];
  return HO_OK;
}

int ho_get_boxes(ho_context* c, float* out) {
  if (!c || !out) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  CK(cudaMemcpyAsync(out, c->d_box, c->n_elem * 6 * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "read boxes");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return HO_OK;
}

int ho_get_hull_boxes(ho_context* c, float* out, float* face_out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (out)
    CK(cudaMemcpyAsync(out, c->d_hull, c->n_elem * 6 * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "read");
  if (face_out)
    CK(cudaMemcpyAsync(face_out, c->d_fbox, c->n_elem * ho::kFaceBoxFloats * sizeof(float), cudaMemcpyDeviceToHost,
                       c->stream),
       "read");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return HO_OK;
}

int ho_render_device(ho_context* c, const ho_camera* cam, const float* iso, int n_iso, int W, int H,
                     int iso_zero_disables, uint8_t* rgb_dev, ho_hit* hits_dev, void* stream) {
  if (!c) return HO_ERR_ARG;
  if (!cam) return fail(c, HO_ERR_ARG, "camera is NULL");
  int rc = check_iso(c, iso, n_iso);
  if (rc) return rc;
  if (W <= 0 || H <= 0) return fail(c, HO_ERR_ARG, "image size must be positive");
  if (static_cast<int64_t>(W) * H * n_iso > (int64_t(1) << 31)) return fail(c, HO_ERR_RANGE, "too many rays");
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  ho::TraceArgs a;
  camera_basis(*cam, W, H, a);
  a.n_iso = n_iso;
  for (int i = 0; i < n_iso; ++i) {
    a.iso[i] = iso[i];
    if (!(iso_zero_disables && iso[i] == 0.0f)) a.iso_on_mask |= 1u << i;
  }
  a.rgb = rgb_dev;
  a.hits = hits_dev;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  CK(cudaMemsetAsync(c->d_stats, 0, sizeof(ho::DevStats), s), "reset stats");
  rc = ho::launch_trace(c, a, s);
  if (rc) return cuda_fail(c, rc, "trace kernel");
  return mark_call_done(c, s);
}

int ho_render_tile_device(ho_context* c, const ho_camera* cam, const float* iso, int n_iso, int W, int H, int x0,
                          int y0, int tile_w, int tile_h, int iso_zero_disables, uint8_t* rgb_dev, ho_hit* hits_dev,
                          void* stream) {
  if (!c) return HO_ERR_ARG;
  if (!cam) return fail(c, HO_ERR_ARG, "camera is NULL");
  int rc = check_iso(c, iso, n_iso);
  if (rc) return rc;
  if (W <= 0 || H <= 0 || tile_w <= 0 || tile_h <= 0) return fail(c, HO_ERR_ARG, "image and tile sizes must be positive");
  if (x0 < 0 || y0 < 0 || x0 > W - tile_w || y0 > H - tile_h)
    return fail(c, HO_ERR_RANGE, "the tile must lie inside the W x H image");
  if (static_cast<int64_t>(tile_w) * tile_h * n_iso > (int64_t(1) << 31)) return fail(c, HO_ERR_RANGE, "too many rays");
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  ho::TraceArgs a;
  camera_basis(*cam, W, H, a);
  a.width = tile_w;
  a.height = tile_h;
  a.x0 = x0;
  a.y0 = y0;
  a.full_w = W;
  a.full_h = H;
  a.n_iso = n_iso;
  for (int i = 0; i < n_iso; ++i) {
    a.iso[i] = iso[i];
    if (!(iso_zero_disables && iso[i] == 0.0f)) a.iso_on_mask |= 1u << i;
  }
  a.rgb = rgb_dev;
  a.hits = hits_dev;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  CK(cudaMemsetAsync(c->d_stats, 0, sizeof(ho::DevStats), s), "reset stats");
  rc = ho::launch_trace(c, a, s);
  if (rc) return cuda_fail(c, rc, "trace kernel");
  return mark_call_done(c, s);
}

int ho_render_tile(ho_context* c, const ho_camera* cam, const float* iso, int n_iso, int W, int H, int x0, int y0,
                   int tile_w, int tile_h, int iso_zero_disables, uint8_t* rgb_out, ho_hit* hits_out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  int rc = check_iso(c, iso, n_iso);
  if (rc) return rc;
  if (tile_w <= 0 || tile_h <= 0) return fail(c, HO_ERR_ARG, "image and tile sizes must be positive");
  const size_t nq = static_cast<size_t>(tile_w) * tile_h * n_iso;
  if (rgb_out && (rc = ensure_buf(c, c->d_rgb, c->rgb_cap, nq * 3, "cudaMalloc(rgb)"))) return rc;
  if (hits_out && (rc = ensure_buf(c, c->d_hits, c->hits_cap, nq, "cudaMalloc(hits)"))) return rc;
  rc = ho_render_tile_device(c, cam, iso, n_iso, W, H, x0, y0, tile_w, tile_h, iso_zero_disables,
                             rgb_out ? c->d_rgb : nullptr, hits_out ? c->d_hits : nullptr, c->stream);
  if (rc) return rc;
  if (rgb_out) CK(cudaMemcpyAsync(rgb_out, c->d_rgb, nq * 3, cudaMemcpyDeviceToHost, c->stream), "read image");
  if (hits_out)
    CK(cudaMemcpyAsync(hits_out, c->d_hits, nq * sizeof(ho_hit), cudaMemcpyDeviceToHost, c->stream), "read hits");
  return read_stats(c);
}

int ho_render_views_device(ho_context* c, int n_views, const ho_camera* cams, const int32_t* widths,
                           const int32_t* heights, const float* isovalues, const int32_t* n_isos, int iso_zero_disables,
                           uint8_t* rgb_dev, ho_hit* hits_dev, int64_t* offsets_out, void* stream) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (n_views < 1 || n_views > (1 << 20)) return fail(c, HO_ERR_RANGE, "n_views must be in [1, 2^20]");
  if (!cams || !widths || !heights || !isovalues || !n_isos) return fail(c, HO_ERR_ARG, "null argument");
  std::vector<ho::ViewDesc> views(n_views);
  int64_t total = 0;
  for (int v = 0; v < n_views; ++v) {
    if (widths[v] <= 0 || heights[v] <= 0) return fail(c, HO_ERR_ARG, "image size must be positive");
    if (n_isos[v] < 1 || n_isos[v] > 8) return fail(c, HO_ERR_RANGE, "n_isos must be in [1, 8]");
    ho::TraceArgs a;
    camera_basis(cams[v], widths[v], heights[v], a);
    ho::ViewDesc& d = views[v];
    d.cam.origin = make_float3(a.origin[0], a.origin[1], a.origin[2]);
    d.cam.llc = make_float3(a.llc[0], a.llc[1], a.llc[2]);
    d.cam.horiz = make_float3(a.horiz[0], a.horiz[1], a.horiz[2]);
    d.cam.vert = make_float3(a.vert[0], a.vert[1], a.vert[2]);
    d.cam.width = widths[v];
    d.cam.height = heights[v];
    d.cam.x0 = d.cam.y0 = 0;
    d.cam.full_w = widths[v];
    d.cam.full_h = heights[v];
    d.q0 = total;
    d.n_iso = n_isos[v];
    d.iso_on_mask = 0;
    for (int i = 0; i < 8; ++i) {
      d.iso[i] = i < n_isos[v] ? isovalues[8 * v + i] : 0.f;
      if (i < n_isos[v] && !(iso_zero_disables && d.iso[i] == 0.0f)) d.iso_on_mask |= 1u << i;
    }
    if (offsets_out) offsets_out[v] = total;
    total += static_cast<int64_t>(widths[v]) * heights[v] * n_isos[v];
  }
  if (offsets_out) offsets_out[n_views] = total;
  if (total > (int64_t(1) << 31)) return fail(c, HO_ERR_RANGE, "too many rays");
  int rc;
  if ((rc = ensure_buf(c, c->d_views, c->views_cap, views.size() * sizeof(ho::ViewDesc), "cudaMalloc(views)")))
    return rc;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  CK(cudaMemcpyAsync(c->d_views, views.data(), views.size() * sizeof(ho::ViewDesc), cudaMemcpyHostToDevice, s),
     "upload views");
  ho::TraceArgs a;
  a.views = reinterpret_cast<const ho::ViewDesc*>(c->d_views);
  a.n_views = n_views;
  a.n_queries_views = total;
  a.n_iso = 1;
  a.rgb = rgb_dev;
  a.hits = hits_dev;
  CK(cudaMemsetAsync(c->d_stats, 0, sizeof(ho::DevStats), s), "reset stats");
  rc = ho::launch_trace(c, a, s);
  if (rc) return cuda_fail(c, rc, "trace kernel");
  return mark_call_done(c, s);
}

int ho_render_views(ho_context* c, int n_views, const ho_camera* cams, const int32_t* widths, const int32_t* heights,
                    const float* isovalues, const int32_t* n_isos, int iso_zero_disables, uint8_t* rgb_out,
                    ho_hit* hits_out, int64_t* offsets_out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (n_views < 1 || !widths || !heights || !n_isos) return fail(c, HO_ERR_ARG, "null argument or no views");
  int64_t total = 0;
  for (int v = 0; v < n_views; ++v)
    total += static_cast<int64_t>(std::max(widths[v], 0)) * std::max(heights[v], 0) * std::max(n_isos[v], 0);
  const size_t nq = static_cast<size_t>(total);
  int rc;
  if (rgb_out && (rc = ensure_buf(c, c->d_rgb, c->rgb_cap, nq * 3, "cudaMalloc(rgb)"))) return rc;
  if (hits_out && (rc = ensure_buf(c, c->d_hits, c->hits_cap, nq, "cudaMalloc(hits)"))) return rc;
  rc = ho_render_views_device(c, n_views, cams, widths, heights, isovalues, n_isos, iso_zero_disables,
                              rgb_out ? c->d_rgb : nullptr, hits_out ? c->d_hits : nullptr, offsets_out, c->stream);
  if (rc) return rc;
  if (rgb_out) CK(cudaMemcpyAsync(rgb_out, c->d_rgb, nq * 3, cudaMemcpyDeviceToHost, c->stream), "read images");
  if (hits_out)
    CK(cudaMemcpyAsync(hits_out, c->d_hits, nq * sizeof(ho_hit), cudaMemcpyDeviceToHost, c->stream), "read hits");
  return read_stats(c);
}

int ho_render(ho_context* c, const ho_camera* cam, const float* iso, int n_iso, int W, int H, int iso_zero_disables,
              uint8_t* rgb_out, ho_hit* hits_out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  int rc = check_iso(c, iso, n_iso);
  if (rc) return rc;
  if (W <= 0 || H <= 0) return fail(c, HO_ERR_ARG, "image size must be positive");
  const size_t nq = static_cast<size_t>(W) * H * n_iso;
  if (rgb_out && (rc = ensure_buf(c, c->d_rgb, c->rgb_cap, nq * 3, "cudaMalloc(rgb)"))) return rc;
  if (hits_out && (rc = ensure_buf(c, c->d_hits, c->hits_cap, nq, "cudaMalloc(hits)"))) return rc;
  rc = ho_render_device(c, cam, iso, n_iso, W, H, iso_zero_disables, rgb_out ? c->d_rgb : nullptr,
                        hits_out ? c->d_hits : nullptr, c->stream);
  if (rc) return rc;
  if (rgb_out) CK(cudaMemcpyAsync(rgb_out, c->d_rgb, nq * 3, cudaMemcpyDeviceToHost, c->stream), "read image");
  if (hits_out)
    CK(cudaMemcpyAsync(hits_out, c->d_hits, nq * sizeof(ho_hit), cudaMemcpyDeviceToHost, c->stream), "read hits");
  return read_stats(c);
}

int ho_intersect_device(ho_context* c, int64_t n, const float* rays_dev, float iso, int iso_enabled, ho_hit* out_dev,
                        void* stream) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (n < 0 || n > (int64_t(1) << 31)) return fail(c, HO_ERR_RANGE, "ray count out of range");
  if (n > 0 && (!rays_dev || !out_dev)) return fail(c, HO_ERR_ARG, "null buffer");
  ho::TraceArgs a;
  a.rays = rays_dev;
  a.n_rays = n;
  a.n_iso = 1;
  a.iso[0] = iso;
  a.iso_on_mask = iso_enabled ? 1u : 0u;
  a.hits = out_dev;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  CK(cudaMemsetAsync(c->d_stats, 0, sizeof(ho::DevStats), s), "reset stats");
  if (n == 0) return mark_call_done(c, s);
  const int rc = ho::launch_trace(c, a, s);
  if (rc) return cuda_fail(c, rc, "trace kernel");
  return mark_call_done(c, s);
}

int ho_intersect(ho_context* c, int64_t n, const float* rays, float iso, int iso_enabled, ho_hit* out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (n < 0) return fail(c, HO_ERR_ARG, "n must be >= 0");
  if (n > 0 && (!rays || !out)) return fail(c, HO_ERR_ARG, "null buffer");
  int rc;
  if ((rc = ensure_buf(c, c->d_rays, c->rays_cap, static_cast<size_t>(n) * 6, "cudaMalloc(rays)"))) return rc;
  if ((rc = ensure_buf(c, c->d_hits, c->hits_cap, static_cast<size_t>(n), "cudaMalloc(hits)"))) return rc;
  if (n > 0)
    CK(cudaMemcpyAsync(c->d_rays, rays, n * 6 * sizeof(float), cudaMemcpyHostToDevice, c->stream), "upload rays");
  rc = ho_intersect_device(c, n, c->d_rays, iso, iso_enabled, c->d_hits, c->stream);
  if (rc) return rc;
  if (n > 0) CK(cudaMemcpyAsync(out, c->d_hits, n * sizeof(ho_hit), cudaMemcpyDeviceToHost, c->stream), "read hits");
  return read_stats(c);
}

namespace {
// rays from 6 arrays of n (ox, oy, oz, dx, dy, dz) to n records of 6 floats
__global__ void soa_to_rays_kernel(const float* __restrict__ soa, int64_t n, float* __restrict__ rays) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int k = 0; k < 6; ++k) rays[6 * i + k] = soa[k * n + i];
}
}  // namespace

int ho_intersect_soa(ho_context* c, int64_t n, const float* ray_soa, float iso, int iso_enabled, ho_hit* out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (n < 0) return fail(c, HO_ERR_ARG, "n must be >= 0");
  if (n > 0 && (!ray_soa || !out)) return fail(c, HO_ERR_ARG, "null buffer");
  int rc;
  // the upload in the second half of the ray buffer, the records in the first
  if ((rc = ensure_buf(c, c->d_rays, c->rays_cap, static_cast<size_t>(n) * 12, "cudaMalloc(rays)"))) return rc;
  if ((rc = ensure_buf(c, c->d_hits, c->hits_cap, static_cast<size_t>(n), "cudaMalloc(hits)"))) return rc;
  if (n > 0) {
    float* soa = c->d_rays + static_cast<size_t>(n) * 6;
    CK(cudaMemcpyAsync(soa, ray_soa, n * 6 * sizeof(float), cudaMemcpyHostToDevice, c->stream), "upload rays");
    soa_to_rays_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, c->stream>>>(soa, n, c->d_rays);
    CK(cudaGetLastError(), "soa_to_rays_kernel");
  }
  rc = ho_intersect_device(c, n, c->d_rays, iso, iso_enabled, c->d_hits, c->stream);
  if (rc) return rc;
  if (n > 0) CK(cudaMemcpyAsync(out, c->d_hits, n * sizeof(ho_hit), cudaMemcpyDeviceToHost, c->stream), "read hits");
  return read_stats(c);
}

int ho_path_trace_device(ho_context* c, const ho_camera* cam, const float* iso, int n_iso, int W, int H, int spp,
                         int max_depth, uint64_t seed, int iso_zero_disables, uint8_t* rgb_dev, int64_t* rays_traced,
                         void* stream) {
  if (!c) return HO_ERR_ARG;
  if (!cam || !rgb_dev) return fail(c, HO_ERR_ARG, "null argument");
  int rc = check_iso(c, iso, n_iso);
  if (rc) return rc;
  if (W <= 0 || H <= 0) return fail(c, HO_ERR_ARG, "image size must be positive");
  if (spp < 1 || spp > 65536) return fail(c, HO_ERR_RANGE, "spp must be in [1, 65536]");
  if (max_depth < 1 || max_depth > 64) return fail(c, HO_ERR_RANGE, "max_depth must be in [1, 64]");
  const int64_t npix = static_cast<int64_t>(W) * H;
  if (npix > (int64_t(1) << 30) || npix * spp > (int64_t(1) << 32))
    return fail(c, HO_ERR_RANGE, "too many paths (W * H * spp must stay below 2^32)");
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  ho::TraceArgs a;
  camera_basis(*cam, W, H, a);
  const ho::CamArgs ca = ho::cam_args(a);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  int64_t rays = 0;
  ho_stats totals{};
  for (int k = 0; k < n_iso; ++k) {
    const bool on = !(iso_zero_disables && iso[k] == 0.0f);
    rc = ho::path_trace(c, ca, iso[k], on, spp, max_depth, seed, rgb_dev + static_cast<size_t>(k) * npix * 3, &rays,
                        &totals, s);
    if (rc < 0) return rc;
    if (rc > 0) return cuda_fail(c, rc, "path tracing");
  }
  if (rays_traced) *rays_traced = rays;
  // ho_get_stats reports the whole call: the engine's counters summed over
  // every bounce and isovalue
  c->last = totals;
  c->stats_frozen = true;
  return HO_OK;
}

int ho_path_trace(ho_context* c, const ho_camera* cam, const float* iso, int n_iso, int W, int H, int spp,
                  int max_depth, uint64_t seed, int iso_zero_disables, uint8_t* rgb_out, int64_t* rays_traced) {
  if (!c) return HO_ERR_ARG;
  if (!rgb_out) return fail(c, HO_ERR_ARG, "rgb_out is NULL");
  int rc = check_iso(c, iso, n_iso);
  if (rc) return rc;
  if (W <= 0 || H <= 0) return fail(c, HO_ERR_ARG, "image size must be positive");
  const size_t bytes = static_cast<size_t>(W) * H * n_iso * 3;
  if ((rc = ensure_buf(c, c->d_rgb, c->rgb_cap, bytes, "cudaMalloc(rgb)"))) return rc;
  rc = ho_path_trace_device(c, cam, iso, n_iso, W, H, spp, max_depth, seed, iso_zero_disables, c->d_rgb, rays_traced,
                            c->stream);
  if (rc) return rc;
  CK(cudaMemcpyAsync(rgb_out, c->d_rgb, bytes, cudaMemcpyDeviceToHost, c->stream), "read image");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return HO_OK;
}

int ho_hit_residuals(ho_context* c, int64_t n, const float* rays, const ho_hit* hits, double* out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (n < 0) return fail(c, HO_ERR_ARG, "n must be >= 0");
  if (n == 0) return HO_OK;
  if (!rays || !hits || !out) return fail(c, HO_ERR_ARG, "null buffer");
  for (int64_t i = 0; i < n; ++i)
    if ((hits[i].kind == HO_HIT_FACE || hits[i].kind == HO_HIT_ISO) && (hits[i].elem < 0 || hits[i].elem >= c->n_elem))
      return fail(c, HO_ERR_RANGE, "hit " + std::to_string(i) + " names no element of the scene");
  if (c->n_elem == 0) {  // no hexahedron hits: every residual is 0
    std::memset(out, 0, static_cast<size_t>(n) * 2 * sizeof(double));
    return HO_OK;
  }
  int rc;
  if ((rc = ensure_buf(c, c->d_rays, c->rays_cap, static_cast<size_t>(n) * 6, "cudaMalloc(rays)"))) return rc;
  if ((rc = ensure_buf(c, c->d_hits, c->hits_cap, static_cast<size_t>(n), "cudaMalloc(hits)"))) return rc;
  double* d_out = nullptr;
  CK(cudaMalloc(&d_out, static_cast<size_t>(n) * 2 * sizeof(double)), "cudaMalloc(residuals)");
  cudaError_t e = cudaMemcpyAsync(c->d_rays, rays, n * 6 * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_hits, hits, n * sizeof(ho_hit), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = static_cast<cudaError_t>(ho::launch_residuals(c, n, c->d_rays, c->d_hits, d_out, c->stream));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d_out, n * 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_out);
  CK(e, "hit residuals");
  return HO_OK;
}

int ho_set_option(ho_context* c, int option, int64_t value) {
  if (!c) return HO_ERR_ARG;
  switch (option) {
    case HO_OPT_GRAPH:
      if (value != 0 && value != 1) return fail(c, HO_ERR_RANGE, "HO_OPT_GRAPH takes 0 or 1");
      c->use_graph = value == 1;
      return HO_OK;
    case HO_OPT_ROUNDS:
      if (value < 1 || value > 256) return fail(c, HO_ERR_RANGE, "HO_OPT_ROUNDS must be in [1, 256]");
      c->round_count = static_cast<int>(value);
      return HO_OK;
    case HO_OPT_ROUND_CHUNK:
      if (value < 1 || value > 4096) return fail(c, HO_ERR_RANGE, "HO_OPT_ROUND_CHUNK must be in [1, 4096]");
      c->round_chunk = static_cast<int>(value);
      return HO_OK;
    case HO_OPT_FP64_CHECK:
      if (value != 0 && value != 1) return fail(c, HO_ERR_RANGE, "HO_OPT_FP64_CHECK takes 0 or 1");
      c->fp64_check = value == 1;
      return HO_OK;
    case HO_OPT_TIME_ROUNDS:
      if (value != 0 && value != 1) return fail(c, HO_ERR_RANGE, "HO_OPT_TIME_ROUNDS takes 0 or 1");
      c->time_rounds = value == 1;
      return HO_OK;
    case HO_OPT_TENSOR:
      if (value != 0 && value != 1) return fail(c, HO_ERR_RANGE, "HO_OPT_TENSOR takes 0 or 1");
      c->use_tc = value == 1;
      return HO_OK;
    case HO_OPT_TAIL:
      if (value < 0 || value > 256) return fail(c, HO_ERR_RANGE, "HO_OPT_TAIL must be in [0, 256]");
      c->tail_after = static_cast<int>(value);
      return HO_OK;
    case HO_OPT_GPU_FIT:
      if (value < -1 || value > 1) return fail(c, HO_ERR_RANGE, "HO_OPT_GPU_FIT takes -1, 0 or 1");
      c->gpu_fit = static_cast<int>(value);
      return HO_OK;
    case HO_OPT_WARM_CAP:
      if (value < 1 || value > 50) return fail(c, HO_ERR_RANGE, "HO_OPT_WARM_CAP must be in [1, 50]");
      c->warm_cap = static_cast<int>(value);
      return HO_OK;
    default:
      return fail(c, HO_ERR_ARG, "unknown option " + std::to_string(option));
  }
}

int ho_get_option(ho_context* c, int option, int64_t* value) {
  if (!c || !value) return HO_ERR_ARG;
  switch (option) {
    case HO_OPT_GRAPH: *value = c->use_graph ? 1 : 0; return HO_OK;
    case HO_OPT_FP64_CHECK: *value = c->fp64_check ? 1 : 0; return HO_OK;
    case HO_OPT_TIME_ROUNDS: *value = c->time_rounds ? 1 : 0; return HO_OK;
    case HO_OPT_TENSOR: *value = c->use_tc ? 1 : 0; return HO_OK;
    case HO_OPT_TAIL: *value = c->tail_after; return HO_OK;
    case HO_OPT_GPU_FIT: *value = c->gpu_fit; return HO_OK;
    case HO_OPT_LAST_FIT_GPU: *value = c->last_fit_gpu ? 1 : 0; return HO_OK;
    case HO_OPT_ROUNDS: *value = c->round_count; return HO_OK;
    case HO_OPT_WARM_CAP: *value = c->warm_cap; return HO_OK;
    case HO_OPT_ROUND_CHUNK:
      *value = c->round_chunk > 0 ? c->round_chunk : ho::round_batch_default(c->N > 0 ? c->N : 2, c->use_tc);
      return HO_OK;
    default: return fail(c, HO_ERR_ARG, "unknown option " + std::to_string(option));
  }
}

int ho_autotune(ho_context* c, const ho_camera* cam, const float* iso, int n_iso, int W, int H, int iso_zero_disables,
                int64_t* chunk_out, int64_t* candidates_out, float* ms_out) {
  if (!c) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (!cam || !chunk_out) return fail(c, HO_ERR_ARG, "null argument");
  int rc = check_iso(c, iso, n_iso);
  if (rc) return rc;
  if (W <= 0 || H <= 0) return fail(c, HO_ERR_ARG, "image size must be positive");
  const size_t nq = static_cast<size_t>(W) * H * n_iso;
  if ((rc = ensure_buf(c, c->d_rgb, c->rgb_cap, nq * 3, "cudaMalloc(rgb)"))) return rc;
  const int slots = ho::round_batch_default(c->N, c->use_tc);
  const int64_t cand[HO_AUTOTUNE_N] = {slots / 2, slots, 2 * slots, 4 * slots, 8 * slots};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  CK(cudaEventCreate(&ev0), "cudaEventCreate");
  CK(cudaEventCreate(&ev1), "cudaEventCreate");
  const int keep = c->round_chunk;
  float best_ms = 0.f;
  int64_t best = keep;
  for (int k = 0; k < HO_AUTOTUNE_N && rc == HO_OK; ++k) {
    c->round_chunk = static_cast<int>(cand[k]);
    float ms = 0.f;
    for (int rep = 0; rep < 2 && rc == HO_OK; ++rep) {
      if (rep == 1 && cudaEventRecord(ev0, c->stream) != cudaSuccess) rc = fail(c, HO_ERR_CUDA, "event record");
      if (rc == HO_OK) rc = ho_render_device(c, cam, iso, n_iso, W, H, iso_zero_disables, c->d_rgb, nullptr, c->stream);
      if (rc == HO_OK && rep == 1) {
        if (cudaEventRecord(ev1, c->stream) != cudaSuccess || cudaEventSynchronize(ev1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess)
          rc = fail(c, HO_ERR_CUDA, "event timing");
      }
    }
    if (rc != HO_OK) break;
    if (ms_out) ms_out[k] = ms;
    if (candidates_out) candidates_out[k] = cand[k];
    if (k == 0 || ms < best_ms) {
      best_ms = ms;
      best = cand[k];
    }
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  c->round_chunk = rc == HO_OK ? static_cast<int>(best) : keep;
  if (rc != HO_OK) return rc;
  *chunk_out = best;
  return read_stats(c);
}

int ho_set_mode(ho_context* c, int mode) {
  if (!c) return HO_ERR_ARG;
  if (mode == HO_MODE_PLAIN || mode == HO_MODE_BATCHED) {
    c->mode = mode;
    return HO_OK;
  }
  if (mode == HO_MODE_LEARNED) {
    if (!c->mlp.trained) return fail(c, HO_ERR_STATE, "learned mode needs a trained or loaded network");
    c->mode = mode;
    return HO_OK;
  }
  return fail(c, HO_ERR_ARG, "unknown mode");
}

// ---- learned mode ----------------------------------------------------------
namespace {
const int kLayerIn[4] = {ho::kMlpIn, ho::kMlpHidden, ho::kMlpHidden, ho::kMlpHidden};
const int kLayerInPad[4] = {ho::kMlpInPad, ho::kMlpHidden, ho::kMlpHidden, ho::kMlpHidden};
const int kLayerOut[4] = {ho::kMlpHidden, ho::kMlpHidden, ho::kMlpHidden, ho::kMlpOut};

// flat layout W1[48][128] b1 W2[128][128] b2 W3 b3 W4[128][8] b4 -> padded per-layer host arrays
void unflatten(const float* flat, std::vector<std::vector<float>>& W, std::vector<std::vector<float>>& b) {
  W.assign(4, {});
  b.assign(4, {});
  size_t o = 0;
  for (int l = 0; l < 4; ++l) {
    W[l].assign(static_cast<size_t>(kLayerInPad[l]) * kLayerOut[l], 0.f);
    for (int i = 0; i < kLayerIn[l]; ++i)
      for (int j = 0; j < kLayerOut[l]; ++j) W[l][static_cast<size_t>(i) * kLayerOut[l] + j] = flat[o++];
    b[l].assign(flat + o, flat + o + kLayerOut[l]);
    o += kLayerOut[l];
  }
}

void flatten(const std::vector<std::vector<float>>& W, const std::vector<std::vector<float>>& b, float* flat) {
  size_t o = 0;
  for (int l = 0; l < 4; ++l) {
    for (int i = 0; i < kLayerIn[l]; ++i)
      for (int j = 0; j < kLayerOut[l]; ++j) flat[o++] = W[l][static_cast<size_t>(i) * kLayerOut[l] + j];
    for (int j = 0; j < kLayerOut[l]; ++j) flat[o++] = b[l][j];
  }
}

int upload_params(ho_context* c, const float* flat) {
  std::vector<std::vector<float>> W, b;
  unflatten(flat, W, b);
  const float* Wp[4] = {W[0].data(), W[1].data(), W[2].data(), W[3].data()};
  const float* bp[4] = {b[0].data(), b[1].data(), b[2].data(), b[3].data()};
  const int rc = c->mlp.set_params(Wp, bp, c->stream);
  if (rc) return cuda_fail(c, rc, "network parameters");
  CK(cudaStreamSynchronize(c->stream), "sync");
  return HO_OK;
}

int download_params(ho_context* c, float* flat, bool grads) {
  std::vector<std::vector<float>> W(4), b(4);
  for (int l = 0; l < 4; ++l) {
    W[l].resize(static_cast<size_t>(kLayerInPad[l]) * kLayerOut[l]);
    b[l].resize(kLayerOut[l]);
    CK(cudaMemcpyAsync(W[l].data(), grads ? c->mlp.gW[l] : c->mlp.W[l], W[l].size() * sizeof(float),
                       cudaMemcpyDeviceToHost, c->stream), "read parameters");
    CK(cudaMemcpyAsync(b[l].data(), grads ? c->mlp.gb[l] : c->mlp.b[l], b[l].size() * sizeof(float),
                       cudaMemcpyDeviceToHost, c->stream), "read parameters");
  }
  CK(cudaStreamSynchronize(c->stream), "sync");
  flatten(W, b, flat);
  return HO_OK;
}

void to_bf16_rows(const float* X, int64_t n, std::vector<uint16_t>& out) {
  out.assign(static_cast<size_t>(n) * ho::kMlpInPad, 0);
  for (int64_t r = 0; r < n; ++r)
    for (int j = 0; j < ho::kMlpIn; ++j) {
      uint32_t u;
      std::memcpy(&u, &X[r * ho::kMlpIn + j], 4);
      const uint32_t lsb = (u >> 16) & 1u;  // round to nearest even
      out[static_cast<size_t>(r) * ho::kMlpInPad + j] = static_cast<uint16_t>((u + 0x7FFFu + lsb) >> 16);
    }
}
}  // namespace

int ho_mlp_init(ho_context* c, uint64_t seed) {
  if (!c) return HO_ERR_ARG;
  int rc = ensure_device(c);
  if (rc) return rc;
  std::vector<float> flat(ho::kMlpParams, 0.f);
  ho::Pcg64 g(seed, 11);
  size_t o = 0;
  for (int l = 0; l < 4; ++l) {
    const double lim = std::sqrt(6.0 / (kLayerIn[l] + kLayerOut[l]));  // Glorot uniform
    for (int i = 0; i < kLayerIn[l] * kLayerOut[l]; ++i) flat[o++] = static_cast<float>((2.0 * g.uniform() - 1.0) * lim);
    o += kLayerOut[l];  // zero biases
  }
  return upload_params(c, flat.data());
}

int ho_mlp_set_params(ho_context* c, const float* params) {
  if (!c || !params) return HO_ERR_ARG;
  int rc = ensure_device(c);
  if (rc) return rc;
  rc = upload_params(c, params);
  if (rc) return rc;
  c->mlp.trained = true;
  return HO_OK;
}

int ho_mlp_get_params(ho_context* c, float* params) {
  if (!c || !params) return HO_ERR_ARG;
  if (!c->mlp.ready) return fail(c, HO_ERR_STATE, "no network");
  return download_params(c, params, false);
}

int ho_mlp_forward(ho_context* c, const float* X, int64_t n, float* Y) {
  if (!c || (n > 0 && (!X || !Y))) return HO_ERR_ARG;
  if (!c->mlp.ready) return fail(c, HO_ERR_STATE, "no network");
  if (n == 0) return HO_OK;
  std::vector<uint16_t> xb;
  to_bf16_rows(X, n, xb);
  void* dx = nullptr;
  float* dy = nullptr;
  CK(cudaMalloc(&dx, xb.size() * 2), "cudaMalloc");
  CK(cudaMalloc(&dy, static_cast<size_t>(n) * ho::kMlpOut * sizeof(float)), "cudaMalloc");
  CK(cudaMemcpyAsync(dx, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice, c->stream), "upload");
  const int rc = ho::mlp_infer(c->mlp.dev(), dx, n, nullptr, 1, dy, c->stream, 152);
  if (rc) return cuda_fail(c, rc, "network forward");
  CK(cudaMemcpyAsync(Y, dy, static_cast<size_t>(n) * ho::kMlpOut * sizeof(float), cudaMemcpyDeviceToHost, c->stream),
     "read");
  CK(cudaStreamSynchronize(c->stream), "sync");
  cudaFree(dx);
  cudaFree(dy);
  return HO_OK;
}

int ho_mlp_grad(ho_context* c, const float* X, const float* T, const uint8_t* valid, int n, float* loss,
                float* grads) {
  if (!c || !X || !T || !valid || n <= 0 || !loss || !grads) return HO_ERR_ARG;
  if (!c->mlp.ready) return fail(c, HO_ERR_STATE, "no network");
  std::vector<uint16_t> xb;
  to_bf16_rows(X, n, xb);
  void* dx = nullptr;
  float *dt = nullptr, *dl = nullptr;
  uint8_t* dv = nullptr;
  CK(cudaMalloc(&dx, xb.size() * 2), "cudaMalloc");
  CK(cudaMalloc(&dt, static_cast<size_t>(n) * ho::kMlpOut * sizeof(float)), "cudaMalloc");
  CK(cudaMalloc(&dv, n), "cudaMalloc");
  CK(cudaMalloc(&dl, sizeof(float)), "cudaMalloc");
  CK(cudaMemcpyAsync(dx, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice, c->stream), "upload");
  CK(cudaMemcpyAsync(dt, T, static_cast<size_t>(n) * ho::kMlpOut * sizeof(float), cudaMemcpyHostToDevice, c->stream),
     "upload");
  CK(cudaMemcpyAsync(dv, valid, n, cudaMemcpyHostToDevice, c->stream), "upload");
  int nv = 0;
  for (int i = 0; i < n; ++i) nv += valid[i] ? 1 : 0;
  const int rc = c->mlp.forward_backward(n, dx, dt, dv, nv, dl, c->stream);
  if (rc) return cuda_fail(c, rc, "network backward");
  CK(cudaMemcpyAsync(loss, dl, sizeof(float), cudaMemcpyDeviceToHost, c->stream), "read");
  const int r2 = download_params(c, grads, true);
  cudaFree(dx);
  cudaFree(dt);
  cudaFree(dv);
  cudaFree(dl);
  return r2;
}

int ho_learn_samples(ho_context* c, int64_t n, uint64_t seed, float* X, float* T, uint8_t* valid) {
  if (!c || n <= 0 || !X || !T || !valid) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (c->n_elem == 0) return fail(c, HO_ERR_STATE, "the network learns hexahedra; the scene has none");
  void* dx = nullptr;
  float* dt = nullptr;
  uint8_t* dv = nullptr;
  CK(cudaMalloc(&dx, static_cast<size_t>(n) * ho::kMlpInPad * 2), "cudaMalloc");
  CK(cudaMalloc(&dt, static_cast<size_t>(n) * ho::kMlpOut * sizeof(float)), "cudaMalloc");
  CK(cudaMalloc(&dv, n), "cudaMalloc");
  int rc = ho::launch_datagen(c->N, c->d_rec, c->d_box, c->d_desc, c->n_elem, n, seed, dx, dt, dv, c->stream);
  if (rc) return cuda_fail(c, rc, "training-pair kernel");
  std::vector<uint16_t> xb(static_cast<size_t>(n) * ho::kMlpInPad);
  CK(cudaMemcpyAsync(xb.data(), dx, xb.size() * 2, cudaMemcpyDeviceToHost, c->stream), "read");
  CK(cudaMemcpyAsync(T, dt, static_cast<size_t>(n) * ho::kMlpOut * sizeof(float), cudaMemcpyDeviceToHost, c->stream),
     "read");
  CK(cudaMemcpyAsync(valid, dv, n, cudaMemcpyDeviceToHost, c->stream), "read");
  CK(cudaStreamSynchronize(c->stream), "sync");
  for (int64_t r = 0; r < n; ++r)
    for (int j = 0; j < ho::kMlpIn; ++j) {
      const uint32_t u = static_cast<uint32_t>(xb[static_cast<size_t>(r) * ho::kMlpInPad + j]) << 16;
      std::memcpy(&X[r * ho::kMlpIn + j], &u, 4);
    }
  cudaFree(dx);
  cudaFree(dt);
  cudaFree(dv);
  return HO_OK;
}

int ho_train_mlp(ho_context* c, int64_t n_samples, int steps, int batch, float lr, uint64_t seed, float* losses) {
  if (!c || n_samples <= 0 || steps <= 0 || batch <= 0 || batch > 65536) return HO_ERR_ARG;
  if (!c->built) return fail(c, HO_ERR_STATE, "call ho_build_bvh first");
  if (c->n_elem == 0) return fail(c, HO_ERR_STATE, "the network learns hexahedra; the scene has none");
  if (!c->mlp.ready) {
    const int rc = ho_mlp_init(c, seed);
    if (rc) return rc;
  }
  void* dx = nullptr;
  float* dt = nullptr;
  uint8_t* dv = nullptr;
  CK(cudaMalloc(&dx, static_cast<size_t>(n_samples) * ho::kMlpInPad * 2), "cudaMalloc(training inputs)");
  CK(cudaMalloc(&dt, static_cast<size_t>(n_samples) * ho::kMlpOut * sizeof(float)), "cudaMalloc(training targets)");
  CK(cudaMalloc(&dv, n_samples), "cudaMalloc");
  int rc = ho::launch_datagen(c->N, c->d_rec, c->d_box, c->d_desc, c->n_elem, n_samples, seed, dx, dt, dv, c->stream);
  if (rc) return cuda_fail(c, rc, "training-pair kernel");
  std::vector<float> hist;
  rc = c->mlp.train(dx, dt, dv, n_samples, steps, batch, lr, seed, hist, c->stream);
  cudaFree(dx);
  cudaFree(dt);
  cudaFree(dv);
  if (rc) return cuda_fail(c, rc, "training");
  if (losses) std::memcpy(losses, hist.data(), hist.size() * sizeof(float));
  return HO_OK;
}

// Checkpoint: "HOMLP001", int32 parameter count, FP32 master parameters, then
// their BF16 copy (round to nearest even) in the same flat order.
int ho_mlp_save(ho_context* c, const char* path) {
  if (!c || !path) return HO_ERR_ARG;
  if (!c->mlp.ready) return fail(c, HO_ERR_STATE, "no network");
  std::vector<float> flat(ho::kMlpParams);
  int rc = download_params(c, flat.data(), false);
  if (rc) return rc;
  std::vector<uint16_t> hb(flat.size());
  for (size_t i = 0; i < flat.size(); ++i) {
    uint32_t u;
    std::memcpy(&u, &flat[i], 4);
    hb[i] = static_cast<uint16_t>((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(c, HO_ERR_IO, std::string("cannot write ") + path);
  const int32_t cnt = ho::kMlpParams;
  bool ok = std::fwrite("HOMLP001", 1, 8, f) == 8 && std::fwrite(&cnt, 4, 1, f) == 1 &&
            std::fwrite(flat.data(), 4, flat.size(), f) == flat.size() &&
            std::fwrite(hb.data(), 2, hb.size(), f) == hb.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? HO_OK : fail(c, HO_ERR_IO, std::string("short write to ") + path);
}

int ho_mlp_load(ho_context* c, const char* path) {
  if (!c || !path) return HO_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(c, HO_ERR_IO, std::string("cannot read ") + path);
  char magic[8];
  int32_t cnt = 0;
  std::vector<float> flat(ho::kMlpParams);
  const bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "HOMLP001", 8) == 0 &&
                  std::fread(&cnt, 4, 1, f) == 1 && cnt == ho::kMlpParams &&
                  std::fread(flat.data(), 4, flat.size(), f) == flat.size();
  std::fclose(f);
  if (!ok) return fail(c, HO_ERR_PARSE, std::string("not a network checkpoint: ") + path);
  return ho_mlp_set_params(c, flat.data());
}

int ho_get_stats(ho_context* c, ho_stats* out) {
  if (!c || !out) return HO_ERR_ARG;
  if (c->stream && c->d_stats && !c->stats_frozen) {
    const int rc = read_stats(c);
    if (rc && rc != HO_ERR_DEVICE) return rc;
  }
  *out = c->last;
  return HO_OK;
}

int ho_save_ppm(const uint8_t* rgb, int W, int H, const char* path) {
  if (!rgb || !path || W <= 0 || H <= 0) return HO_ERR_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return HO_ERR_IO;
  std::fprintf(f, "P6\n%d %d\n255\n", W, H);
  const size_t n = static_cast<size_t>(W) * H * 3;
  const bool ok = std::fwrite(rgb, 1, n, f) == n;
  std::fclose(f);
  return ok ? HO_OK : HO_ERR_IO;
}

// PNG (ISO/IEC 15948): 8-bit RGB, no interlace, every row with filter type
// 0, the image data a zlib stream (RFC 1950) of stored deflate blocks
// (RFC 1951, uncompressed), chunk CRC-32 over type and data.
namespace {
struct CrcTable {
  uint32_t v[256];
  CrcTable() {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t x = i;
      for (int k = 0; k < 8; ++k) x = (x & 1u) ? 0xedb88320u ^ (x >> 1) : x >> 1;
      v[i] = x;
    }
  }
};

uint32_t png_crc(const uint8_t* p, size_t n, uint32_t c = 0xffffffffu) {
  static const CrcTable crc;  // built once, thread-safe
  const uint32_t* table = crc.v;
  for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xffu] ^ (c >> 8);
  return c;
}

void put_be32(std::vector<uint8_t>& out, uint32_t v) {
  for (int s = 24; s >= 0; s -= 8) out.push_back(static_cast<uint8_t>(v >> s));
}

void put_chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put_be32(out, static_cast<uint32_t>(data.size()));
  const size_t at = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  put_be32(out, png_crc(out.data() + at, out.size() - at) ^ 0xffffffffu);
}
}  // namespace

int ho_save_png(const uint8_t* rgb, int W, int H, const char* path) {
  if (!rgb || !path || W <= 0 || H <= 0) return HO_ERR_ARG;
  const size_t row = static_cast<size_t>(W) * 3;
  if (row + 1 > 0x7fffffffu / static_cast<size_t>(H)) return HO_ERR_RANGE;
  // raw scanlines: filter byte 0, then the row
  std::vector<uint8_t> raw;
  raw.reserve((row + 1) * H);
  for (int y = 0; y < H; ++y) {
    raw.push_back(0);
    raw.insert(raw.end(), rgb + y * row, rgb + (y + 1) * row);
  }
  std::vector<uint8_t> z;
  z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
  z.push_back(0x78);  // deflate, 32 KB window
  z.push_back(0x01);  // no dictionary, fastest; (0x78 << 8 | 0x01) % 31 == 0
  uint32_t a = 1, b = 0;  // Adler-32
  for (size_t at = 0; at < raw.size() || at == 0;) {
    const size_t n = std::min<size_t>(65535, raw.size() - at);
    const bool last = at + n == raw.size();
    z.push_back(last ? 1 : 0);  // BFINAL, BTYPE 00 (stored)
    z.push_back(static_cast<uint8_t>(n));
    z.push_back(static_cast<uint8_t>(n >> 8));
    z.push_back(static_cast<uint8_t>(~n));
    z.push_back(static_cast<uint8_t>(~n >> 8));
    z.insert(z.end(), raw.begin() + at, raw.begin() + at + n);
    for (size_t i = at; i < at + n; ++i) {
      a = (a + raw[i]) % 65521u;
      b = (b + a) % 65521u;
    }
    at += n;
    if (last) break;
  }
  put_be32(z, b << 16 | a);
  std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<uint8_t> ihdr;
  put_be32(ihdr, static_cast<uint32_t>(W));
  put_be32(ihdr, static_cast<uint32_t>(H));
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8 bits, RGB, deflate, filter set 0, no interlace
  put_chunk(out, "IHDR", ihdr);
  put_chunk(out, "IDAT", z);
  put_chunk(out, "IEND", {});
  FILE* f = std::fopen(path, "wb");
  if (!f) return HO_ERR_IO;
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  return (std::fclose(f) == 0 && ok) ? HO_OK : HO_ERR_IO;
}

}  // extern "C"
