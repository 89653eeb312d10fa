// Host-side types of the renderer: the context behind the C ABI, the scene as
// the caller gave it, and the helpers shared by the host translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "ho_layout.h"
#include "ho_mlp.h"
#include "horender.h"

namespace ho {

// Scene as supplied (ho_add_hexes / loader / generator): same layout as the
// reference's Scene hex buffers (FEM-AABB/raytracer.h:65-96), one entry per
// element, coefficients FP32.
// Prisms, quads and curved triangles, in the order they were added; the
// device keeps them kind by kind (prisms, quads, triangles), each kind in
// this order.
struct HostPrims {
  std::vector<int32_t> kind;      // 0 prism, 1 quad, 2 triangle
  std::vector<float> verts;       // n*18 (6 / 4 / 3 vertices used)
  std::vector<uint32_t> gmodes;   // n*3 (prism x, y, z; quad / triangle x, y, 0)
  std::vector<uint32_t> fmodes;   // n*3
  std::vector<int64_t> goff;      // n, -1 = linear geometry
  std::vector<int64_t> foff;      // n, -1 = no field
  std::vector<float> geom;        // x, y, z blocks per curved primitive
  std::vector<float> field;
  int64_t size() const { return static_cast<int64_t>(kind.size()); }
};

struct HostScene {
  HostPrims prims;
  std::vector<float> corners;     // n*24, XML vertex order
  std::vector<uint32_t> gmodes;   // n*3 (0,0,0 = trilinear from corners)
  std::vector<uint32_t> fmodes;   // n*3
  std::vector<int64_t> goff;      // n, -1 = trilinear
  std::vector<int64_t> foff;      // n, -1 = no field
  std::vector<float> geom;
  std::vector<float> field;
  int64_t size() const { return static_cast<int64_t>(goff.size()); }
};

// GLL nodes on [-1,1], ascending, computed in FP64.
std::vector<double> gll_nodes(int n);
// Modified-A mode i and its derivative at x, FP64.
double mod_a(int i, double x);
double mod_a_prime(int i, double x);
// Inverse of the n x n matrix V[row][col] = phi_col(nodes[row]) (FP64).
bool modal_vandermonde_inverse(const std::vector<double>& nodes, std::vector<double>& inv);
// Tensor-product modal fit of nodal values (i fastest) on GLL nodes.
void tensor_modal_fit(int n, const std::vector<double>& vinv, const double* nodal, double* modal);

// Seeded synthetic scene generation (appends to hs).
int generate_synthetic(const ho_synth_params& p, HostScene& hs, std::string& err);

// Largest modes count over geometry and field (trilinear counts as 2).
int scene_max_modes(const HostScene& hs);
// Pack the scene into per-element records of record_floats(N) floats (x, y,
// z geometry blocks then the field block, rows padded to row_stride(N)),
// zero-padded to N modes per direction.
// Trilinear elements become their exact N = 2 modal form. flags[e] bit 0:
// has field; bit 1: trilinear (box rule of FEM-AABB/high_order.h:59-76);
// own[e]: the element's own geometry modes (box sample count).
void pack_records(const HostScene& hs, int N, std::vector<float>& rec, std::vector<uint32_t>& flags,
                  std::vector<int32_t>& own);

// Cube order of an element: its largest geometry or field modes count per
// direction (trilinear: 2).
int element_order(const HostScene& hs, int64_t e);
// Every element's record at its own order, back to back: off[e] is its
// first float, order[e] its modes per direction (same block layout as
// pack_records at N = order[e]).
void pack_compact(const HostScene& hs, std::vector<float>& rec, std::vector<int64_t>& off, std::vector<uint8_t>& order);

// 1-D change of basis Modified-A -> Bernstein on [a,b] for n modes:
// phi_i(x) = sum_k M[i*n+k] * B_k((x-a)/(b-a)).
void modal_to_bernstein(int n, double a, double b, std::vector<double>& M);

// PCG-XSL-RR 128/64 generator (published PCG64 algorithm).
struct Pcg64 {
  unsigned __int128 state, inc;
  Pcg64(uint64_t seed, uint64_t stream);
  uint64_t next();
  double uniform();  // [0,1), 53 bits
};

// Tensor-product modal fit of elements' nodal geometry (FP64 values on GLL
// nodes, i fastest, one block of nx*ny*nz values per component) into FP32
// Modified-A coefficients written to (*dst)[dst_off ...]: the component
// blocks back to back, coefficient index (k*ny + j)*nx + i. A fitter may
// hold jobs back and write them in finish(); dst must stay alive (it may be
// reallocated) until then.
class ModalFitter {
 public:
  virtual ~ModalFitter() = default;
  virtual bool add(const double* nodal, int comps, int nx, int ny, int nz, std::vector<float>* dst, int64_t dst_off) = 0;
  virtual bool finish() = 0;
  virtual const char* error() const { return "modal fit failed"; }
};
// The host fitter (FP64, per element, immediately).
std::unique_ptr<ModalFitter> make_host_fitter();
// The GPU fitter (ho_fit.cu): jobs gathered in pinned host memory, fitted in
// batches by one CTA per element (FP64 sum factorisation), on `device`.
std::unique_ptr<ModalFitter> make_gpu_fitter(int device);

// fitter: the geometry's modal fit (nullptr: the host fitter).
int load_xml_fld(const std::string& xml, const std::string& fld, HostScene& hs, std::string& err,
                 ModalFitter* fitter = nullptr);
// ASCII VTK XML unstructured-grid hexahedra (trilinear, no field), appended.
int load_vtu(const std::string& path, HostScene& hs, std::string& err);

}  // namespace ho

namespace ho {
// Scratch of the element-major intersection rounds, grown on demand.
struct RoundBufs {
  void* state = nullptr;     // per queue item
  size_t state_cap = 0;
  void* pairs = nullptr;     // gathered + element-sorted pairs
  size_t pairs_cap = 0;
  int32_t* pelem = nullptr;
  size_t pelem_cap = 0;
  uint32_t* prank = nullptr;
  size_t prank_cap = 0;
  void* batches = nullptr;
  size_t batches_cap = 0;
  uint32_t* ecount = nullptr;  // per element
  size_t ecount_cap = 0;
  uint32_t* eoff = nullptr;
  size_t eoff_cap = 0;
  uint32_t* tile_sums = nullptr;  // per 4096 elements, for the offsets' scan
  size_t tile_sums_cap = 0;
  unsigned* ctr = nullptr;   // pairs, batches, next batch, failed FP64 checks
  size_t ctr_cap = 0;
  uint32_t* fail = nullptr;  // queue items whose hit failed the FP64 check
  size_t fail_cap = 0;
};
}  // namespace ho

struct ho_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int mode = HO_MODE_BATCHED;
  ho::HostScene hs;
  bool built = false;

  // device scene
  int N = 0;
  int64_t n_elem = 0;
  float* d_rec = nullptr;         // n_elem * record_floats(N)
  // mixed-order scenes: every element's record at its own order (the round
  // kernels read these; everything else reads d_rec)
  float* d_crec = nullptr;
  int64_t* d_coff = nullptr;      // n_elem, float offset of each record in d_crec
  uint8_t* d_cord = nullptr;      // n_elem, modes per direction of each record
  uint32_t orders = 0;            // bit n: some element has order n
  float* d_box = nullptr;         // n_elem * 6 padded sampled boxes
  float* d_hull = nullptr;        // n_elem * 6 Bernstein hull boxes
  float* d_fbox = nullptr;        // n_elem * 36 face hull boxes
  uint32_t* d_flags = nullptr;    // n_elem
  int32_t* d_own = nullptr;       // n_elem
  ho::BNode* d_nodes = nullptr;   // max(1, n_elem - 1)
  int64_t n_nodes = 0;
  int bvh_depth = 0;
  float bounds[6] = {0, 0, 0, 0, 0, 0};
  int64_t device_bytes = 0;

  // prisms, quads and curved triangles (ho_prim.cu)
  int64_t n_prims = 0;
  void* d_prims = nullptr;        // n_prims PrimRec, kind-major
  float* d_pgeom = nullptr;
  float* d_pfield = nullptr;
  float* d_pbox = nullptr;        // n_prims * 6
  ho::BNode* d_pnodes = nullptr;  // max(1, n_prims - 1)
  int64_t n_pnodes = 0;
  int pbvh_depth = 0;
  int64_t prim_counts[3] = {0, 0, 0};
  ho_hit* d_phits = nullptr;      // hits of calls that asked for none (the primitive pass needs them)
  size_t phits_cap = 0;
  cudaEvent_t prim_events[2] = {nullptr, nullptr};  // HO_OPT_TIME_ROUNDS: around the primitive pass
  bool prim_timed = false;        // the last trace call recorded them

  ho::DevStats* d_stats = nullptr;
  ho_stats last{};
  // Recorded on the caller's stream at the end of a *_device call, so that
  // reading the counters and timing events over the context's own stream
  // waits for that call's kernels.
  cudaEvent_t call_done = nullptr;
  bool call_done_pending = false;

  // render scratch
  ho_hit* d_hits = nullptr;
  size_t hits_cap = 0;
  uint8_t* d_rgb = nullptr;
  size_t rgb_cap = 0;
  float* d_rays = nullptr;
  size_t rays_cap = 0;
  uint8_t* d_views = nullptr;     // view table of a multi-view call
  size_t views_cap = 0;
  // learned mode
  ho::Mlp mlp;
  float* d_desc = nullptr;        // n_elem * 48 element descriptors
  float* d_pred = nullptr;        // network outputs, [queue item][kPredK][8]
  int32_t* d_cand = nullptr;      // elements the predictions belong to
  size_t pred_cap = 0;
  int32_t* d_work = nullptr;      // query queue of the intersect pass
  float2* d_kbuf = nullptr;       // first ordered candidates per queued query
  uint8_t* d_kovf = nullptr;
  size_t work_cap = 0;
  unsigned* d_qctr = nullptr;     // [0] queue length, [1] next item
  ho::RoundBufs rounds;
  // batched / learned engine options (ho_set_option)
  int round_chunk = 0;       // pairs per element batch (0: the kernel's pair slots)
  int warm_cap = 4;          // round kernel: iterations of a warm-started solve before its cold restart
  int round_count = 16;      // rounds enqueued before the completion check (at most)
  int tail_after = 4;        // rounds before the warp-per-ray tail finishes every ray (0: no tail)
  int gpu_fit = -1;          // loader's modal fit: -1 on the GPU when one is present, 0 host, 1 GPU
  bool last_fit_gpu = false; // the last load fitted on the GPU
  int64_t launches = 0;      // kernels enqueued by the last trace call
  bool stats_frozen = false; // last holds a path-tracing call's totals (not refreshed from the device)
  bool time_rounds = false;  // event pairs around each round's intersection launches
  std::vector<cudaEvent_t> round_events;
  int round_events_used = 0;  // events recorded by the last trace call
  int rounds_needed = 0;     // non-empty rounds of the previous batched / learned call
  bool use_graph = true;     // run a call's launches as one CUDA graph
  bool fp64_check = true;    // FP64 residual check + plain fallback of the hits
  bool use_tc = false;       // tensor-core round kernel for orders up to kTcMaxModes
  bool graph_warm = false;   // the first call of a context runs direct
  cudaGraphExec_t graph_exec = nullptr;
  bool last_graph = false;
  void* h_pinned = nullptr;
  size_t pinned_cap = 0;
};

namespace ho {
// Kernel launchers (ho_build.cu / ho_trace.cu). Return cudaError_t as int.
int launch_setup(ho_context* c);
int build_lbvh(ho_context* c);
// LBVH over n device boxes (lo xyz, hi xyz); leaf aux bits from d_flags
// (nullable). Allocates *nodes_out (max(1, n - 1) nodes).
int build_tree(const float* d_box, const uint32_t* d_flags, int64_t n, cudaStream_t s, BNode** nodes_out,
               int64_t* n_nodes_out, int* depth_out, float bounds[6]);
struct TraceArgs {
  // camera mode (rays == nullptr): pixel-centre rays of a pinhole camera
  float origin[3], llc[3], horiz[3], vert[3];
  int width = 0, height = 0;
  int x0 = 0, y0 = 0;           // a tile of the full_w x full_h image (0: the
  int full_w = 0, full_h = 0;   // whole image, full = width, height)
  const float* rays = nullptr;  // explicit rays: n*6 floats on the device
  int64_t n_rays = 0;
  float iso[8];
  int n_iso = 0;
  uint32_t iso_on_mask = 0;     // bit i: isovalue i enabled
  const ViewDesc* views = nullptr;  // multi-view call: device table
  int n_views = 0;
  int64_t n_queries_views = 0;  // total queries of the views
  ho_hit* hits = nullptr;       // optional
  uint8_t* rgb = nullptr;       // optional (camera mode)
};
int launch_trace(ho_context* c, const TraceArgs& a, cudaStream_t s);
// The kernels' camera of a camera-mode call.
inline CamArgs cam_args(const TraceArgs& a) {
  CamArgs c;
  c.origin = make_float3(a.origin[0], a.origin[1], a.origin[2]);
  c.llc = make_float3(a.llc[0], a.llc[1], a.llc[2]);
  c.horiz = make_float3(a.horiz[0], a.horiz[1], a.horiz[2]);
  c.vert = make_float3(a.vert[0], a.vert[1], a.vert[2]);
  c.width = a.width;
  c.height = a.height;
  c.x0 = a.x0;
  c.y0 = a.y0;
  c.full_w = a.full_w > 0 ? a.full_w : a.width;
  c.full_h = a.full_h > 0 ? a.full_h : a.height;
  return c;
}
// Path tracing of one image at one isovalue (ho_path.cu); returns a
// cudaError_t, or a negative HO_ status from the engine (message set).
int path_trace(ho_context* c, const CamArgs& cam, float iso, bool iso_on, int spp, int max_depth, uint64_t seed,
               uint8_t* rgb, int64_t* rays_traced, ho_stats* totals, cudaStream_t s);
// Primitive scene upload, boxes and tree (ho_prim.cu); frees the old one.
int prims_build(ho_context* c);
void prims_free(ho_context* c);
// The primitive pass over the queries of a trace call: each query's hit is
// replaced by a nearer primitive hit. fresh: the hexahedra were not traced
// (a scene without them); every query is written.
// stats: device counters for the traversal status (nullptr: the context's).
int launch_prims(ho_context* c, const TraceArgs& a, ho_hit* hits, bool fresh, DevStats* stats, cudaStream_t s);
// The FP64 check's residuals for caller-given hits (ho_rounds.cu).
int launch_residuals(ho_context* c, int64_t n, const float* rays, const ho_hit* hits, double* out, cudaStream_t s);
}  // namespace ho
