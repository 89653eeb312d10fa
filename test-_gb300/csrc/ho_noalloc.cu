// Allocation-free ray queries: ho_intersect_device_noalloc.
//
// Who needs it: callers that are not allowed to call the CUDA allocator at
// query time — a host application that owns all device memory through its
// own pool and forbids libraries from calling cudaMalloc/cudaFree, or a
// real-time loop where the device-wide synchronisation that cudaFree implies
// would stall other work. The regular entry points grow per-context scratch
// buffers with cudaMalloc on demand; this one never allocates.
//
// How: the batched pipeline's scratch (ray queue, per-ray candidate lists,
// queue counters, work counters) lives in the file-scope device array
// g_noalloc_scratch below, sized for kNoAllocMaxRays rays per call (about
// 2.3 MB). Every GPU that loads the library's device code holds this array
// until the process exits; with CUDA's lazy module loading it is placed on a
// device when the first call there looks its address up. The scene itself
// must already be on the device (ho_build_bvh), and the caller supplies the
// ray and hit buffers.
//
// The host cannot use g_noalloc_scratch's name as a device address; the
// device address is looked up with cudaGetSymbolAddress once per device, with
// that device current, on the first call on that device. Make that first call
// before any stream capture.
//
// All calls share the one array, which keeps the previous call's contents:
// the counters are cleared at the start of every call, and calls whose GPU
// work overlaps (two streams, or two host threads) race on the array and
// corrupt each other's results — serialise them.
//
// What it runs: the miss-culling classify pass, then the warp-per-ray
// intersection kernel (isect_kernel) in batched form with cold-start Newton,
// whatever ho_set_mode chose; then the primitive pass when the scene has
// prisms, quads or triangles. It skips the round engine's FP64 residual check
// and plain-solver fallback (their ray lists would need more scratch), so its
// hits carry the FP32 solvers' own stopping rules (|u - iso| < 1e-5 at an
// isosurface root, face residual < 1e-4) without the FP64 confirmation.
// Its counters live in the scratch array, so ho_get_stats does not report
// this call; a ray whose tree walk met the stack limit is flagged
// HO_FLAG_INCOMPLETE in its own hit.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "ho_host.h"
#include "ho_trace.cuh"

namespace ho {

__global__ void __launch_bounds__(256) classify_kernel(TraceParams P, int64_t n_queries);

constexpr int64_t kNoAllocMaxRays = HO_NOALLOC_MAX_RAYS;

// byte layout of the scratch array
constexpr size_t kNaStats = 0;                                         // DevStats
constexpr size_t kNaCounters = 512;                                    // queue length, next item
constexpr size_t kNaWork = 768;                                        // int32 per ray
constexpr size_t kNaKbuf = kNaWork + 4 * kNoAllocMaxRays;              // float2 x kCandK per ray
constexpr size_t kNaKovf = kNaKbuf + 8 * kCandK * kNoAllocMaxRays;     // uint8 per ray
constexpr size_t kNaBytes = kNaKovf + kNoAllocMaxRays;
static_assert(sizeof(DevStats) <= kNaCounters - kNaStats, "stats slot too small");
static_assert(kNaKbuf % 16 == 0, "candidate lists must be 16-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (made current by the caller).
cudaError_t scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_addr[device]);
  return cudaSuccess;
}
}  // namespace

}  // namespace ho

extern "C" int ho_intersect_device_noalloc(ho_context* c, int64_t n, const float* rays_dev, float iso,
                                           int iso_enabled, ho_hit* out_dev, void* stream) {
  using namespace ho;
  if (!c) return HO_ERR_ARG;
  if (!c->built) {
    c->err = "call ho_build_bvh first";
    return HO_ERR_STATE;
  }
  if (n < 0 || n > kNoAllocMaxRays) {
    c->err = "ho_intersect_device_noalloc: n = " + std::to_string(n) + " rays, the limit is " +
             std::to_string(kNoAllocMaxRays) + " per call";
    return HO_ERR_RANGE;
  }
  if (n > 0 && (!rays_dev || !out_dev)) {
    c->err = "null buffer";
    return HO_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(c->device);
  unsigned char* base = nullptr;
  if (e == cudaSuccess) e = scratch_address(c->device, &base);
  if (e != cudaSuccess) {
    c->err = std::string("scratch set-up: ") + cudaGetErrorString(e);
    return HO_ERR_CUDA;
  }
  // an empty call touches nothing on the device, so it cannot clear the
  // counters under another call still in flight
  if (n == 0) return HO_OK;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  // the counters and work totals must start at zero; the lists are written
  // before they are read
  e = cudaMemsetAsync(base, 0, kNaWork, s);
  if (e != cudaSuccess) {
    c->err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(e);
    return HO_ERR_CUDA;
  }
  TraceParams P;
  P.nodes = c->d_nodes;
  P.rec = c->d_rec;
  P.fbox = c->d_fbox;
  P.box = c->d_box;
  P.flags = c->d_flags;
  P.rays = rays_dev;
  P.n_rays = n;
  P.cam = CamArgs{};
  for (int i = 0; i < 8; ++i) P.iso[i] = 0.f;
  P.iso[0] = iso;
  P.n_iso = 1;
  P.iso_on_mask = iso_enabled ? 1u : 0u;
  P.views = nullptr;
  P.n_views = 0;
  P.hits = out_dev;
  P.rgb = nullptr;
  P.stats = reinterpret_cast<DevStats*>(base + kNaStats);
  P.qcount = reinterpret_cast<unsigned*>(base + kNaCounters);
  P.qnext = P.qcount + 1;
  P.work = reinterpret_cast<int32_t*>(base + kNaWork);
  P.kbuf = reinterpret_cast<float2*>(base + kNaKbuf);
  P.kovf = base + kNaKovf;
  P.desc = nullptr;
  P.cand_e = nullptr;
  P.pred = nullptr;
  P.pred_items = 0;
  P.fp64 = 0;
  if (c->n_elem == 0) {  // primitives only
    TraceArgs a;
    a.rays = rays_dev;
    a.n_rays = n;
    a.n_iso = 1;
    a.iso[0] = iso;
    a.iso_on_mask = P.iso_on_mask;
    e = static_cast<cudaError_t>(launch_prims(c, a, out_dev, true, P.stats, s));
    if (e != cudaSuccess) {
      c->err = std::string("primitive kernel: ") + cudaGetErrorString(e);
      return HO_ERR_CUDA;
    }
    return HO_OK;
  }
  classify_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(P, n);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    switch (c->N) {
      case 2: e = launch_n<2>(P, n, n, s, HO_MODE_BATCHED); break;
      case 3: e = launch_n<3>(P, n, n, s, HO_MODE_BATCHED); break;
      case 4: e = launch_n<4>(P, n, n, s, HO_MODE_BATCHED); break;
      case 5: e = launch_n<5>(P, n, n, s, HO_MODE_BATCHED); break;
      case 6: e = launch_n<6>(P, n, n, s, HO_MODE_BATCHED); break;
      case 7: e = launch_n<7>(P, n, n, s, HO_MODE_BATCHED); break;
      case 8: e = launch_n<8>(P, n, n, s, HO_MODE_BATCHED); break;
      case 9: e = launch_n<9>(P, n, n, s, HO_MODE_BATCHED); break;
      default: e = cudaErrorInvalidValue; break;
    }
  }
  if (e == cudaSuccess && c->n_prims > 0) {
    TraceArgs a;
    a.rays = rays_dev;
    a.n_rays = n;
    a.n_iso = 1;
    a.iso[0] = iso;
    a.iso_on_mask = P.iso_on_mask;
    e = static_cast<cudaError_t>(launch_prims(c, a, out_dev, false, P.stats, s));
  }
  if (e != cudaSuccess) {
    c->err = std::string("trace kernels: ") + cudaGetErrorString(e);
    return HO_ERR_CUDA;
  }
  return HO_OK;
}
