// Path tracing with diffuse bounces on top of the batched / learned
// intersection engine (the reference's render loop, FEM-AABB/raytracer.cu:
// 410-476, ray_color 362-406, Lambertian scatter 60-98).
//
// Wavefront form: every sample pass starts one path per pixel; each bounce
// is one call of the intersection engine on the paths still alive (explicit
// rays), then path_scatter_kernel shades misses against the sky, multiplies
// the attenuation by the hit's albedo and writes the scattered rays of the
// surviving paths, compacted. A path that is still alive after max_depth
// intersections contributes black, as in the reference.
//
// Materials as the reference's main.cu:39-41 assigns them: boundary face 0
// of a hex is material 1 (albedo 0.1, 0.2, 0.8), every other hex hit and
// every isosurface hit material 0 (0.5 grey); both Lambertian, no emission.
// Random numbers are counter-based (path, bounce, dimension), so a pass is
// reproducible and independent of the order the engine returns hits in; the
// reference draws from curand with a time seed, so its images are not
// reproducible either way.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "ho_host.h"
#include "ho_trace.cuh"

namespace ho {

// PCG-based integer hash (Jarzynski and Olano, "Hash Functions for GPU
// Rendering", JCGT 2020).
__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
  const uint32_t state = v * 747796405u + 2891336453u;
  const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

// Uniform in [0, 1) from (path key, bounce, dimension): 24 random bits.
__host__ __device__ __forceinline__ float path_u01(uint32_t key, uint32_t bounce, uint32_t dim) {
  const uint32_t h = pcg_hash(pcg_hash(key + pcg_hash(bounce * 8u + dim)) ^ 0x85ebca6bu);
  return static_cast<float>(h >> 8) * (1.0f / 16777216.0f);
}

__host__ __device__ __forceinline__ uint32_t path_key(uint64_t path, uint64_t seed) {
  return pcg_hash(static_cast<uint32_t>(path) ^ pcg_hash(static_cast<uint32_t>(seed) ^ 0x9e3779b9u)) ^
         static_cast<uint32_t>(seed >> 32);
}

// Primary rays of sample pass `sample`: jittered through the pixel
// (u = (x + r0) / W, v = (y + r1) / H), normalised (raytracer.cu:436-447).
__global__ void path_primary_kernel(CamArgs cam, int64_t npix, uint32_t sample, uint64_t seed,
                                    float* __restrict__ rays, float* __restrict__ att, uint32_t* __restrict__ pix,
                                    uint32_t* __restrict__ keys) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const uint32_t key = path_key(static_cast<uint64_t>(i) + static_cast<uint64_t>(npix) * sample, seed);
  const int x = static_cast<int>(i % cam.width), y = static_cast<int>(i / cam.width);
  const float u = (static_cast<float>(x) + path_u01(key, 0u, 0u)) / static_cast<float>(cam.width);
  const float v = (static_cast<float>(y) + path_u01(key, 0u, 1u)) / static_cast<float>(cam.height);
  float3 d = make_float3(cam.llc.x + u * cam.horiz.x + v * cam.vert.x - cam.origin.x,
                         cam.llc.y + u * cam.horiz.y + v * cam.vert.y - cam.origin.y,
                         cam.llc.z + u * cam.horiz.z + v * cam.vert.z - cam.origin.z);
  d = normalize3(d);
  float* r = rays + 6 * i;
  r[0] = cam.origin.x;
  r[1] = cam.origin.y;
  r[2] = cam.origin.z;
  r[3] = d.x;
  r[4] = d.y;
  r[5] = d.z;
  att[3 * i] = att[3 * i + 1] = att[3 * i + 2] = 1.0f;
  pix[i] = static_cast<uint32_t>(i);
  keys[i] = key;
}

// One bounce of every live path, after the engine answered its ray: a miss
// adds attenuation x sky to its pixel (raytracer.cu:398-402); a hit takes the
// material's albedo and, unless this was the path's last allowed
// intersection, continues from the hit point along normal + a uniformly
// random unit vector (raytracer.cu:65-69; the reference's rejection-sampled
// point in the unit ball is normalised there, so only its direction counts).
// Survivors are appended to the output arrays (warp-aggregated).
__global__ void path_scatter_kernel(int64_t n, const float* __restrict__ rays, const ho_hit* __restrict__ hits,
                                    const float* __restrict__ att, const uint32_t* __restrict__ pix,
                                    const uint32_t* __restrict__ keys, uint32_t bounce, int max_depth,
                                    float* __restrict__ accum, float* __restrict__ rays_out,
                                    float* __restrict__ att_out, uint32_t* __restrict__ pix_out,
                                    uint32_t* __restrict__ keys_out, unsigned* __restrict__ n_out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  bool live = false;
  float3 o = make_float3(0.f, 0.f, 0.f), dn = o, a = o;
  uint32_t px = 0, key = 0;
  if (i < n) {
    const float* r = rays + 6 * i;
    const float3 ro = make_float3(r[0], r[1], r[2]), rd = make_float3(r[3], r[4], r[5]);
    const ho_hit h = hits[i];
    a = make_float3(att[3 * i], att[3 * i + 1], att[3 * i + 2]);
    px = pix[i];
    key = keys[i];
    if (h.kind == HO_HIT_MISS) {
      const float3 u = normalize3(rd);
      const float t = 0.5f * (u.y + 1.0f);
      atomicAdd(&accum[3 * px], a.x * ((1.0f - t) + t * 0.5f));
      atomicAdd(&accum[3 * px + 1], a.y * ((1.0f - t) + t * 0.7f));
      atomicAdd(&accum[3 * px + 2], a.z * ((1.0f - t) + t * 1.0f));
    } else {
      const bool blue = h.kind == HO_HIT_FACE && h.face == 0;
      a = make_float3(a.x * (blue ? 0.1f : 0.5f), a.y * (blue ? 0.2f : 0.5f), a.z * (blue ? 0.8f : 0.5f));
      if (static_cast<int>(bounce) + 1 < max_depth) {
        live = true;
        o = make_float3(ro.x + h.t * rd.x, ro.y + h.t * rd.y, ro.z + h.t * rd.z);
        const float z = 1.0f - 2.0f * path_u01(key, bounce + 1u, 0u);
        const float rr = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        float sp, cp;
        sincospif(2.0f * path_u01(key, bounce + 1u, 1u), &sp, &cp);
        dn = make_float3(h.n[0] + rr * cp, h.n[1] + rr * sp, h.n[2] + z);
        // the random vector cancelled the normal: keep the normal (a zero
        // direction has no ray)
        if (dn.x * dn.x + dn.y * dn.y + dn.z * dn.z < 1e-12f) dn = make_float3(h.n[0], h.n[1], h.n[2]);
      }
    }
  }
  const unsigned m = __ballot_sync(0xffffffffu, live);
  if (m == 0u) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(n_out, static_cast<unsigned>(__popc(m)));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!live) return;
  const unsigned k = base + __popc(m & ((1u << lane) - 1u));
  float* ro = rays_out + 6 * static_cast<int64_t>(k);
  ro[0] = o.x;
  ro[1] = o.y;
  ro[2] = o.z;
  ro[3] = dn.x;
  ro[4] = dn.y;
  ro[5] = dn.z;
  att_out[3 * k] = a.x;
  att_out[3 * k + 1] = a.y;
  att_out[3 * k + 2] = a.z;
  pix_out[k] = px;
  keys_out[k] = key;
}

// The image: average over the samples, gamma 2, clamp, 8 bits
// (raytracer.cu:459-475).
__global__ void path_finish_kernel(const float* __restrict__ accum, int64_t npix, int spp, uint8_t* __restrict__ rgb) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const float inv = 1.0f / static_cast<float>(spp);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float v = fminf(1.0f, sqrtf(accum[3 * i + c] * inv));
    rgb[3 * i + c] = static_cast<uint8_t>(255.99f * v);
  }
}

// One image: `spp` passes of one path per pixel, each path traced for up to
// max_depth intersections by the engine on the context (any solver mode),
// isovalue `iso`. rgb: H x W x 3 on the device. Returns a cudaError_t or
// an HO_ status (negative); *rays_traced += the engine's ray queries, and
// *totals += the engine's counters (and the layer's own launches).
int path_trace(ho_context* c, const CamArgs& cam, float iso, bool iso_on, int spp, int max_depth, uint64_t seed,
               uint8_t* rgb, int64_t* rays_traced, ho_stats* totals, cudaStream_t s) {
  const int64_t npix = static_cast<int64_t>(cam.width) * cam.height;
  const size_t n = static_cast<size_t>(npix);
  char* buf = nullptr;
  // two path arrays (rays 24 B, attenuation 12 B, pixel 4 B, key 4 B), hits, accumulator
  const size_t per_path = 2 * (24 + 12 + 4 + 4) + sizeof(ho_hit) + 12;
  cudaError_t e = cudaMalloc(&buf, n * per_path + 16 * 256);
  if (e != cudaSuccess) return int(e);
  char* q = buf;
  auto take = [&](size_t bytes) {
    char* r = q;
    q += (bytes + 255) / 256 * 256;
    return r;
  };
  float* rays[2] = {reinterpret_cast<float*>(take(n * 24)), reinterpret_cast<float*>(take(n * 24))};
  float* att[2] = {reinterpret_cast<float*>(take(n * 12)), reinterpret_cast<float*>(take(n * 12))};
  uint32_t* pix[2] = {reinterpret_cast<uint32_t*>(take(n * 4)), reinterpret_cast<uint32_t*>(take(n * 4))};
  uint32_t* keys[2] = {reinterpret_cast<uint32_t*>(take(n * 4)), reinterpret_cast<uint32_t*>(take(n * 4))};
  ho_hit* hits = reinterpret_cast<ho_hit*>(take(n * sizeof(ho_hit)));
  float* accum = reinterpret_cast<float*>(take(n * 12));
  unsigned* counter = nullptr;
  int rc = 0;
  if ((e = cudaMalloc(&counter, sizeof(unsigned))) != cudaSuccess) rc = int(e);
  if (rc == 0 && (e = cudaMemsetAsync(accum, 0, n * 12, s)) != cudaSuccess) rc = int(e);
  const unsigned grid = static_cast<unsigned>((npix + 255) / 256);
  // the engine's counters summed over its calls (each call restarts them),
  // on top of what *totals holds already
  ho_stats tot = totals ? *totals : ho_stats{};
  auto add = [&](const ho_stats& st) {
    tot.rays += st.rays;
    tot.candidates += st.candidates;
    tot.geom_evals += st.geom_evals;
    tot.map_evals += st.map_evals;
    tot.field_evals += st.field_evals;
    tot.newton_iters += st.newton_iters;
    tot.face_iters += st.face_iters;
    tot.faces_culled += st.faces_culled;
    tot.node_visits += st.node_visits;
    tot.mlp_accepted += st.mlp_accepted;
    tot.mlp_rejected += st.mlp_rejected;
    tot.restarts += st.restarts;
    tot.rounds += st.rounds;
    tot.round_pairs += st.round_pairs;
    tot.solve_steps += st.solve_steps;
    tot.lane_steps += st.lane_steps;
    tot.fp64_checked += st.fp64_checked;
    tot.fp64_failed += st.fp64_failed;
    tot.fp64_failed_after_fallback += st.fp64_failed_after_fallback;
    tot.round_flops += st.round_flops;
    tot.kernel_launches += st.kernel_launches + 1;  // + the scatter kernel
    tot.round_kernel_ns += st.round_kernel_ns;
    tot.round_launches += st.round_launches;
    tot.tail_rays += st.tail_rays;
    tot.prim_candidates += st.prim_candidates;
    tot.prim_iters += st.prim_iters;
    tot.prim_flops += st.prim_flops;
    tot.prim_kernel_ns += st.prim_kernel_ns;
    tot.prim_node_visits += st.prim_node_visits;
    tot.fp64_polished += st.fp64_polished;
    tot.fp64_ties += st.fp64_ties;
    tot.fp64_ties_swapped += st.fp64_ties_swapped;
    tot.grazing_hits += st.grazing_hits;
    tot.graph = st.graph;
    tot.max_modes = st.max_modes;
    tot.status |= st.status;
  };
  for (int sample = 0; sample < spp && rc == 0; ++sample) {
    ++tot.kernel_launches;  // primary rays
    path_primary_kernel<<<grid, 256, 0, s>>>(cam, npix, static_cast<uint32_t>(sample), seed, rays[0], att[0], pix[0],
                                             keys[0]);
    if ((e = cudaGetLastError()) != cudaSuccess) {
      rc = int(e);
      break;
    }
    int64_t live = npix;
    int cur = 0;
    for (int bounce = 0; bounce < max_depth && live > 0; ++bounce) {
      rc = ho_intersect_device(c, live, rays[cur], iso, iso_on ? 1 : 0, hits, s);
      if (rc) break;
      {
        ho_stats st;
        rc = ho_get_stats(c, &st);  // synchronises the stream
        if (rc && rc != HO_ERR_DEVICE) break;
        rc = 0;
        add(st);
      }
      if (rays_traced) *rays_traced += live;
      if ((e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s)) != cudaSuccess) {
        rc = int(e);
        break;
      }
      path_scatter_kernel<<<static_cast<unsigned>((live + 255) / 256), 256, 0, s>>>(
          live, rays[cur], hits, att[cur], pix[cur], keys[cur], static_cast<uint32_t>(bounce), max_depth, accum,
          rays[cur ^ 1], att[cur ^ 1], pix[cur ^ 1], keys[cur ^ 1], counter);
      unsigned next = 0;
      if ((e = cudaGetLastError()) == cudaSuccess)
        e = cudaMemcpyAsync(&next, counter, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        rc = int(e);
        break;
      }
      live = next;
      cur ^= 1;
    }
  }
  if (rc == 0) {
    path_finish_kernel<<<grid, 256, 0, s>>>(accum, npix, spp, rgb);
    if ((e = cudaGetLastError()) != cudaSuccess) rc = int(e);
    ++tot.kernel_launches;
  }
  if (rc == 0 && totals) *totals = tot;
  if (rc == 0 && (e = cudaStreamSynchronize(s)) != cudaSuccess) rc = int(e);
  cudaFree(counter);
  cudaFree(buf);
  return rc;
}

}  // namespace ho
