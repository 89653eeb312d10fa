/*
 * horender — GB300 renderer for curved high-order (spectral/hp) hexahedral
 * meshes and their modal scalar fields.
 *
 * C ABI. Plain pointers and sizes, int status codes, no exceptions across the
 * boundary, caller-owned output buffers. One CUDA stream per context; a
 * context is not thread-safe. Every call returns HO_OK (0) or a negative
 * HO_ERR_* code; ho_last_error() gives the message of the last failure.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the reference project root).
 */
#ifndef HORENDER_H
#define HORENDER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HO_OK 0
#define HO_ERR_ARG (-1)      /* bad argument (null pointer, bad size)            */
#define HO_ERR_CUDA (-2)     /* a CUDA call failed                               */
#define HO_ERR_STATE (-3)    /* call out of order (e.g. render before build)     */
#define HO_ERR_IO (-4)       /* file could not be read or written               */
#define HO_ERR_PARSE (-5)    /* malformed XML / FLD input                       */
#define HO_ERR_NOMEM (-6)    /* device or host allocation failed                */
#define HO_ERR_RANGE (-7)    /* size beyond a documented limit                  */
#define HO_ERR_DEVICE (-8)   /* a kernel reported an internal error status      */

/* Solver modes (ho_set_mode). All three compute the reference's algorithm
 * (same tolerances, same per-candidate policy); they differ in how the work
 * is mapped to the GPU and where Newton starts. */
#define HO_MODE_PLAIN 0      /* one thread per ray, sequential cold-start Newton (the reference's structure) */
#define HO_MODE_LEARNED 1    /* BATCHED + network-predicted Newton starts; plain cold start as fallback     */
#define HO_MODE_BATCHED 2    /* default: miss-culling pass + device queue, then element-major rounds: each
                                round's (ray, element) pairs are bucketed by element and one warp per
                                element batch runs every Newton solve of its pairs from a task queue; a
                                warp per ray finishes the last rays; FP64 residual check + plain fallback */

/* Hit kinds. */
#define HO_HIT_MISS 0
#define HO_HIT_FACE 1
#define HO_HIT_ISO 2
#define HO_HIT_PRISM 3   /* a prism (elem: index among the scene's prisms)    */
#define HO_HIT_QUAD 4    /* a quad (elem: index among the quads)             */
#define HO_HIT_TRI 5     /* a curved triangle (elem: index among the triangles) */

/* ho_hit.flags bits. */
#define HO_FLAG_FALLBACK 1u      /* learned guess rejected, plain solver answered   */
#define HO_FLAG_FP64_FAIL 2u     /* FP64 residual check above tolerance             */
#define HO_FLAG_OVERFLOW 4u      /* candidate list restarted (more than K boxes)     */
#define HO_FLAG_INCOMPLETE 8u    /* the tree walk met its stack limit: candidates may
                                    be missing from this ray's answer                */
#define HO_FLAG_TIE 16u          /* the hit displaced another within 1e-4 in t (one
                                    surface point claimed twice) and the FP64 tie
                                    rule chose between the two (FP64 check on)       */
#define HO_FLAG_GRAZING 32u      /* grazing hit: |cos| of the angle between the ray
                                    and the surface normal below 0.05; a rounding
                                    can move such a hit to a neighbouring face or
                                    element                                          */

typedef struct ho_context ho_context;

/* One ray-query result (48 bytes). kind: HO_HIT_*; elem: element index
 * (-1 on miss); face: 0..5 for boundary-face hits (face table of
 * FEM-AABB/high_order.h:164-184), -1 otherwise; xi: reference coordinates of
 * the hit; n: unit normal facing the ray; u: field value at xi; iters: Newton
 * iterations (inverse map + face) this query spent. */
typedef struct {
  float t;
  int32_t elem;
  int16_t face;
  int16_t kind;
  float xi[3];
  float n[3];
  float u;
  uint32_t flags;
  uint32_t iters;
} ho_hit;

/* Pinhole camera as FEM-AABB/raytracer.h:31-48 (aperture 0: primary rays go
 * through pixel centres, no jitter). vfov in degrees; focus_dist <= 0 means
 * |lookfrom - lookat|. */
typedef struct {
  float lookfrom[3];
  float lookat[3];
  float vup[3];
  float vfov_deg;
  float focus_dist;
} ho_camera;

/* Seeded synthetic scene: an nx*ny*nz grid of hexes over [0,1]^3, GLL
 * geometry nodes displaced by curve_amp*h*sin(2 pi x)sin(2 pi y)sin(2 pi z)
 * (the same scalar added to x, y and z), a field of n_gauss Gaussians
 * (centres U[0,1]^3, sigma U[0.1,0.3], amplitude U[-1,1]) interpolated at
 * the GLL nodes; both fitted to Modified-A modal coefficients in FP64 and
 * stored as FP32. Per-element order P is drawn uniformly from
 * [order_min, order_max] (modes n = P + 1). */
typedef struct {
  int32_t nx, ny, nz;
  int32_t order_min, order_max;
  double curve_amp;
  int32_t n_gauss;
  uint64_t seed;
} ho_synth_params;

typedef struct {
  int64_t n_elem;
  int64_t n_nodes;          /* BVH internal nodes                              */
  int32_t max_modes;        /* largest modes count over geometry and field     */
  int32_t bvh_depth;
  int64_t device_bytes;     /* scene + BVH bytes resident on the device         */
  float bounds[6];          /* scene box (lo xyz, hi xyz) over element boxes    */
  int64_t n_prisms, n_quads, n_tris;  /* other primitives (ho_add_prisms ...) */
} ho_scene_info;

/* Work counters of the last render/intersect call. */
typedef struct {
  uint64_t rays;
  uint64_t candidates;       /* (ray, element) pairs visited                   */
  uint64_t geom_evals;       /* x(xi) + Jacobian evaluations                   */
  uint64_t map_evals;        /* x(xi)-only evaluations                         */
  uint64_t field_evals;      /* u + grad evaluations                           */
  uint64_t newton_iters;     /* inverse-map Newton iterations                  */
  uint64_t face_iters;       /* surface Newton iterations                      */
  uint64_t faces_culled;     /* faces skipped by the exact hull-box test       */
  uint64_t node_visits;      /* BVH node fetches                               */
  uint64_t mlp_accepted;     /* learned guesses that passed the checks         */
  uint64_t mlp_rejected;
  uint64_t restarts;         /* candidate-list overflows                       */
  int32_t max_modes;
  int32_t status;            /* device error status (0 = fine)                 */
  uint64_t phase_cycles[4];  /* warp-per-ray intersect kernel (no-alloc entry):
                                SM cycles per warp in traversal, isosurface
                                scan, bracket refinement, face search         */
  uint64_t rounds;           /* batched/learned: intersection rounds           */
  uint64_t round_pairs;      /* (ray, element) pairs over all rounds           */
  uint64_t solve_steps;      /* loop steps of the round kernel's warps         */
  uint64_t lane_steps;       /* busy lanes summed over those steps: lane use
                                = lane_steps / (32 * solve_steps)             */
  uint64_t graph;            /* 1: the call's launches ran as one CUDA graph   */
  uint64_t fp64_checked;     /* batched/learned: hits re-evaluated in FP64     */
  uint64_t fp64_failed;      /* of those, failed (traced again, plain solver) */
  uint64_t fp64_failed_after_fallback;  /* plain answer failed too (kept,
                                HO_FLAG_FP64_FAIL)                           */
  uint64_t round_flops;      /* batched/learned: algorithmic FP32 flops of the
                                round kernel's evaluations (at each element's
                                order) and Newton solves                     */
  uint64_t kernel_launches;  /* kernels the last trace call launched (graph
                                nodes included)                              */
  uint64_t round_kernel_ns;  /* HO_OPT_TIME_ROUNDS: device time of the round
                                kernels' launches (CUDA events), else 0      */
  uint64_t round_launches;   /* HO_OPT_TIME_ROUNDS: round kernel launches     */
  uint64_t tail_rays;        /* rays finished by the tail (HO_OPT_TAIL)       */
  uint64_t prim_candidates;  /* (query, prism/quad/triangle) pairs visited    */
  uint64_t prim_iters;       /* their Newton / projection iterations          */
  uint64_t prim_flops;       /* algorithmic FP32 flops of the primitive pass  */
  uint64_t prim_kernel_ns;   /* HO_OPT_TIME_ROUNDS: device time of the
                                primitive pass (CUDA events), else 0          */
  uint64_t prim_node_visits; /* primitive-tree nodes visited by that pass     */
  uint64_t fp64_polished;    /* hits whose t, xi and u the FP64 polish moved to
                                the exact root of their defining equations   */
  uint64_t fp64_ties;        /* rays whose best hit displaced another within
                                1e-4 in t (one surface point claimed twice),
                                weighed by the FP64 tie rule                  */
  uint64_t fp64_ties_swapped;  /* of those, rays where the displaced hit won
                                (nearer exact root, or the same point and the
                                lower element / face index)                  */
  uint64_t grazing_hits;     /* hits flagged HO_FLAG_GRAZING                  */
} ho_stats;

/* Replaces: CUDA context/stream set-up and cudaMalloc in FEM-AABB/main.cu:322-511. */
int ho_create(int device, ho_context** out);
/* Replaces: the cudaFree block of FEM-AABB/main.cu:580-597. */
void ho_destroy(ho_context* ctx);
/* Message of the last failed call on this context (never NULL). */
const char* ho_last_error(const ho_context* ctx);

/* Replaces: bool load_xml_fld(xml, fld, Scene&) (FEM-AABB/xml_fld_loader.h:14-16,
 * xml_fld_loader.cpp:16-402). Nektar++ hexahedra with curved edges/faces,
 * composites/expansions; FLD payload ASCII or base64 of zlib / raw deflate /
 * plain FP64 (FP32). Appends to the scene; on error the scene is unchanged.
 * HO_ERR_IO: mesh file unreadable; HO_ERR_PARSE: no vertices or no hexahedra;
 * HO_ERR_RANGE: geometry modes outside [2, 9] or field modes outside [1, 9].
 * A missing or empty FLD file loads the geometry without field. */
int ho_load_xml_fld(ho_context* ctx, const char* xml_path, const char* fld_path);

/* Replaces: bool load_vtu_file(path, Scene&) (FEM-AABB/vtu_loader.h:9,
 * vtu_loader.cpp:156-343). ASCII VTK XML unstructured grid: cells of type
 * 12, 72 or 25 become trilinear hexahedra from their first 8 points, wedges
 * (13, 73, 26) linear prisms from their first 6 and quads (9, 70, 22) linear
 * quads from their first 4, in the file's point order; other cells are
 * skipped; no field. Appends to the scene; on error the scene is unchanged.
 * HO_ERR_IO: file unreadable or empty; HO_ERR_PARSE: no Points/Cells
 * section, no ASCII points/connectivity/types, or no cell of those types. */
int ho_load_vtu(ho_context* ctx, const char* path);

/* Replaces: Scene::add_prism / add_quad / add_curved_tri (FEM-AABB/raytracer.h:
 * 167-300), batched. verts: n*6*3 (prism: quad base 0-3 at t = -1 in the
 * order (-,-), (+,-), (+,+), (-,+) of (r, s), top edge 4-5), n*4*3 (quad:
 * vertex v at r = +-1 by bit 0, s = +-1 by bit 1), n*3*3 (triangle).
 * geom_modes / field_modes: n*3 for prisms (Modified-A in r and s,
 * Modified-B in t), n*2 for quads (A x A) and triangles (A x Modified-B);
 * each in [1, 9]. geom_offsets[i]: float index of primitive i's x block in
 * geom (y, z follow), -1 = linear from the vertices; field_offsets[i]: -1 =
 * no field. Block sizes: quad mx*my; triangle sum_{i<mx} max(my-i, 0);
 * prism my * sum_{i<mx} max(mz-i, 0). Appends; on error nothing is added.
 * The reference traces these with its prism / quad / triangle routines
 * (FEM-AABB/fem/PrismElement.cu, QuadElement.cu, TriElement.cu), prisms
 * without isosurface; so does horender, in a pass after the hexahedra
 * (hits of kind HO_HIT_PRISM / QUAD / TRI). */
int ho_add_prisms(ho_context* ctx, int64_t n, const float* verts, const uint32_t* geom_modes, const float* geom,
                  int64_t geom_len, const int64_t* geom_offsets, const uint32_t* field_modes, const float* field,
                  int64_t field_len, const int64_t* field_offsets);
int ho_add_quads(ho_context* ctx, int64_t n, const float* verts, const uint32_t* geom_modes, const float* geom,
                 int64_t geom_len, const int64_t* geom_offsets, const uint32_t* field_modes, const float* field,
                 int64_t field_len, const int64_t* field_offsets);
int ho_add_tris(ho_context* ctx, int64_t n, const float* verts, const uint32_t* geom_modes, const float* geom,
                int64_t geom_len, const int64_t* geom_offsets, const uint32_t* field_modes, const float* field,
                int64_t field_len, const int64_t* field_offsets);

/* The scene's prisms, quads and triangles as one list, prisms first, then
 * quads, then triangles (each kind in the order added; a hit's elem indexes
 * within its kind): kind (0 prism, 1 quad, 2 triangle), vertices n*18
 * (unused rows zero), modes n*3, offsets into the returned geom / field
 * pools. Any output may be NULL; call with NULL arrays first for the sizes. */
int ho_get_prims(ho_context* ctx, int64_t* n, int32_t* kind, float* verts, uint32_t* geom_modes, float* geom,
                 int64_t* geom_len, int64_t* geom_offsets, uint32_t* field_modes, float* field, int64_t* field_len,
                 int64_t* field_offsets);
/* The primitives' sampled boxes after ho_build_bvh, n*6, in ho_get_prims order. */
int ho_get_prim_boxes(ho_context* ctx, float* out);

/* Replaces: Scene::add_hex (FEM-AABB/raytracer.h:118-166), batched.
 * corners: n*8*3 floats (XML vertex order); geom_modes / field_modes: n*3;
 * geom_offsets[i]: float index of element i's x block in geom (y, z blocks
 * follow, each nx*ny*nz floats), -1 = trilinear from corners;
 * field_offsets[i]: float index into field, -1 = no field. HO_ERR_ARG for a
 * NaN or infinite corner or coefficient (nothing is added). */
int ho_add_hexes(ho_context* ctx, int64_t n, const float* corners, const uint32_t* geom_modes,
                 const float* geom, int64_t geom_len, const int64_t* geom_offsets,
                 const uint32_t* field_modes, const float* field, int64_t field_len,
                 const int64_t* field_offsets);

/* Seeded synthetic scene (no reference counterpart: stands in for the
 * reference's sample meshes at benchmark sizes). Appends to the scene. */
int ho_generate_synthetic(ho_context* ctx, const ho_synth_params* params);

/* Read back the scene as flat arrays (same layout as ho_add_hexes). Call with
 * NULL outputs to get the lengths. */
int ho_get_scene(ho_context* ctx, int64_t* n, float* corners, uint32_t* geom_modes, float* geom,
                 int64_t* geom_len, int64_t* geom_offsets, uint32_t* field_modes, float* field,
                 int64_t* field_len, int64_t* field_offsets);

/* Replaces: Scene::build_bvh() -> BVH::build (FEM-AABB/raytracer.h:338-344,
 * BVH.cu:180-247). Uploads the scene, computes element boxes and builds an
 * LBVH on the device. */
int ho_build_bvh(ho_context* ctx);
int ho_scene_info_get(ho_context* ctx, ho_scene_info* out);
/* Element boxes after ho_build_bvh: n*6 floats (padded sampled box lo, hi). */
int ho_get_boxes(ho_context* ctx, float* out);
/* Rigorous Bernstein hull boxes (n*6) and per-face hull boxes (n*36: 6 faces
 * x lo,hi over u,v in [-1.001,1.001], inflated past the face tolerance);
 * either output may be NULL. No reference counterpart (verification aid). */
int ho_get_hull_boxes(ho_context* ctx, float* hull_out, float* face_out);

/* Many camera views in one call (no reference counterpart; the reference
 * renders one camera per render_kernel launch, FEM-AABB/main.cu:486-511).
 * View v: camera cams[v], widths[v] x heights[v] pixel-centre rays for each
 * of its n_isos[v] (1..8) isovalues isovalues[8*v + 0 .. n_isos[v]-1]. All
 * views' rays run in the same classify pass and rounds. Outputs are laid out
 * view by view, isovalue-major inside a view: view v starts at query
 * offsets_out[v] (n_views + 1 entries, may be NULL), i.e. rgb_out + 3 *
 * offsets_out[v] and hits_out + offsets_out[v]. */
int ho_render_views(ho_context* ctx, int n_views, const ho_camera* cams, const int32_t* widths, const int32_t* heights,
                    const float* isovalues, const int32_t* n_isos, int iso_zero_disables, uint8_t* rgb_out,
                    ho_hit* hits_out, int64_t* offsets_out);
/* Device-buffer form of ho_render_views on the given stream (NULL: the
 * context's stream); returns without synchronising. */
int ho_render_views_device(ho_context* ctx, int n_views, const ho_camera* cams, const int32_t* widths,
                           const int32_t* heights, const float* isovalues, const int32_t* n_isos, int iso_zero_disables,
                           uint8_t* rgb_dev, ho_hit* hits_dev, int64_t* offsets_out, void* stream);

/* Replaces: render_kernel<<<>>> + cudaMemcpy of the framebuffer
 * (FEM-AABB/raytracer.cu:410-476, main.cu:515-543). One primary ray per
 * pixel per isovalue; rgb_out receives n_iso images of H*W*3 bytes, row 0 =
 * bottom of the view as in the reference. iso_zero_disables = 1 gives the
 * reference renderer's rule that isovalue 0 turns the isosurface off
 * (FEM-AABB/raytracer.cu:207). hits_out (optional) receives n_iso*H*W hits. */
int ho_render(ho_context* ctx, const ho_camera* cam, const float* isovalues, int n_iso, int width,
              int height, int iso_zero_disables, uint8_t* rgb_out, ho_hit* hits_out);

/* Device-buffer variant of ho_render: rgb_dev / hits_dev are device pointers
 * (either may be NULL); stream is a cudaStream_t (NULL = the context's). */
int ho_render_device(ho_context* ctx, const ho_camera* cam, const float* isovalues, int n_iso, int width,
                     int height, int iso_zero_disables, uint8_t* rgb_dev, ho_hit* hits_dev, void* stream);

/* One tile of the W x H image of ho_render (no reference counterpart: the
 * reference renders whole images, FEM-AABB/main.cu:515-543; a tile is how
 * several GPUs share one view). The tile_w x tile_h pixels starting at column
 * x0, row y0 get exactly the rays, hits and colours they get in the full
 * render; outputs are laid out like ho_render's for a tile_w x tile_h image.
 * HO_ERR_RANGE when the tile leaves the image. */
int ho_render_tile(ho_context* ctx, const ho_camera* cam, const float* isovalues, int n_iso, int width, int height,
                   int x0, int y0, int tile_w, int tile_h, int iso_zero_disables, uint8_t* rgb_out,
                   ho_hit* hits_out);
/* Device-buffer form of ho_render_tile (stream: a cudaStream_t, NULL = the
 * context's); returns without synchronising. */
int ho_render_tile_device(ho_context* ctx, const ho_camera* cam, const float* isovalues, int n_iso, int width,
                          int height, int x0, int y0, int tile_w, int tile_h, int iso_zero_disables, uint8_t* rgb_dev,
                          ho_hit* hits_dev, void* stream);

/* Replaces: bvh_intersect_device (FEM-AABB/raytracer.cu:102-358) for
 * caller-supplied rays. rays: n*6 floats (origin xyz, direction xyz), host
 * memory; iso_enabled = 0 traces boundary faces only. */
int ho_intersect(ho_context* ctx, int64_t n, const float* rays, float iso, int iso_enabled, ho_hit* out);
/* Device-buffer variant (rays_dev, out_dev on the device). */
int ho_intersect_device(ho_context* ctx, int64_t n, const float* rays_dev, float iso, int iso_enabled,
                        ho_hit* out_dev, void* stream);
/* ho_intersect with the rays as structure of arrays: ray_soa holds 6 arrays
 * of n floats back to back (origin x, y, z, then direction x, y, z), host
 * memory. The same answers as ho_intersect on the same rays. */
int ho_intersect_soa(ho_context* ctx, int64_t n, const float* ray_soa, float iso, int iso_enabled, ho_hit* out);

/* Allocation-free variant of ho_intersect_device (batched mode). No
 * reference counterpart. For callers that may not call the CUDA allocator
 * while querying — an application whose own pool owns all device memory, or a
 * real-time loop that cannot absorb the device-wide synchronisation of
 * cudaFree. Its scratch is one fixed device array (about 2.3 MB, held by every
 * GPU that loads the library's device code until exit; with lazy module
 * loading it becomes resident at the first call on a device) sized for
 * HO_NOALLOC_MAX_RAYS rays per call; larger n fails with HO_ERR_RANGE. Needs ho_build_bvh first; the
 * caller owns rays_dev (n*6 floats) and out_dev (n hits). The first call on a
 * device looks the array's address up; make it before any stream capture.
 * All calls share the array: calls whose GPU work overlaps race.
 * What it runs differs from ho_intersect_device: the miss-culling pass, then
 * the warp-per-ray batched kernel with cold-start Newton whatever the
 * ho_set_mode choice, then the primitive pass. It has no FP64 residual check,
 * no plain-solver fallback and no tail, so its hits meet the FP32 solvers'
 * own stopping rules (|u - iso| < 1e-5 at an isosurface root, face residual
 * < 1e-4) without FP64 confirmation; on the test scenes they equal
 * ho_intersect_device's on at least 99.9% of rays. ho_get_stats does not
 * report this call (its counters sit in the fixed array); a ray whose tree
 * walk met the stack limit carries HO_FLAG_INCOMPLETE in its hit. */
#define HO_NOALLOC_MAX_RAYS 32768
int ho_intersect_device_noalloc(ho_context* ctx, int64_t n, const float* rays_dev, float iso, int iso_enabled,
                                ho_hit* out_dev, void* stream);

/* Solver mode (HO_MODE_*). No reference counterpart: the reference has one.
 * HO_MODE_LEARNED needs a trained (ho_train_mlp) or loaded (ho_mlp_load)
 * network. */
int ho_set_mode(ho_context* ctx, int mode);

/* Options of the batched and learned engine (no reference counterpart).
 * HO_OPT_GRAPH        1 (default): from the second call on, a call's launches
 *                     run as one CUDA graph (patched in place between calls);
 *                     0: direct launches.
 * HO_OPT_ROUNDS       at most this many intersection rounds are enqueued
 *                     before the completion check (default 16, 1..256): a call
 *                     enqueues one more than the previous call needed; rays
 *                     still in flight afterwards get further rounds, one
 *                     read-back each.
 * HO_OPT_FP64_CHECK   1 (default): every hit is re-evaluated in FP64
 *                     (position residual, and field residual for isosurface
 *                     hits). A passing hit is polished: a Newton step on its
 *                     defining equations (FP64 residual, FP32 Jacobian) moves
 *                     t, xi and u to the exact root, within FP32 rounding of
 *                     t (ho_stats.fp64_polished counts them). In batched /
 *                     learned mode a failing hit is traced again by the plain
 *                     solver (HO_FLAG_FALLBACK) and flagged
 *                     HO_FLAG_FP64_FAIL if that fails too; in plain mode it
 *                     is flagged. A hit that displaced another within 1e-4
 *                     in t is weighed against it by the FP64 tie rule
 *                     (HO_FLAG_TIE, ho_stats.fp64_ties). 0: off (the
 *                     solvers' own answers).
 * HO_OPT_ROUND_CHUNK  pairs per element batch of the round kernel (1..4096;
 *                     default: the kernel's pair slots, 20 per warp up to 7
 *                     modes per direction, 12 at 8, 8 at 9, times 4 warps in
 *                     the tensor-core form); ho_autotune picks it.
 * HO_OPT_TENSOR      0 (default): the FP32 CUDA-core round kernel for every
 *                     order; 1: elements of up to 8 modes per direction are
 *                     intersected by the tensor-core round kernel (tcgen05
 *                     TF32 MMAs, split into hi + lo parts, for the first
 *                     contraction; one CTA per element batch). The
 *                     tensor-core form is slower on the benchmark scenes: its
 *                     accumulators take 416 of an SM's 512 tensor-memory
 *                     columns, so one CTA of 4 warps runs per SM, in lockstep,
 *                     and its steps are latency-bound.
 * HO_OPT_TAIL        rounds before the tail (default 4, 0..256; 0: no tail):
 *                     after them, every ray still in flight is finished by
 *                     one warp walking the rest of its candidates (the same
 *                     solves), so the last rays do not wait round by round
 *                     for each round's slowest pair.
 * HO_OPT_GPU_FIT     the loader's modal fit of the element geometry:
 *                     -1 (default) on the GPU when the context's device is
 *                     present, else on the host; 0 host; 1 GPU (an error
 *                     without a device). Both fit in FP64 in the same order.
 * HO_OPT_LAST_FIT_GPU (read only) 1 when the last ho_load_xml_fld fitted on
 *                     the GPU.
 * HO_OPT_WARM_CAP     learned mode, round kernel: Newton iterations a
 *                     network-started inverse map may take before it restarts
 *                     cold (default 4, 1..50). Any value gives the same
 *                     answers (the cold restart is the plain solver); it
 *                     trades iterations of failing warm starts against cold
 *                     restarts.
 * HO_OPT_TIME_ROUNDS  0 (default); 1: a pair of CUDA events brackets each
 *                     round's intersection launches (event nodes of the graph)
 *                     and ho_stats.round_kernel_ns / round_launches report
 *                     their device time.
 * HO_ERR_ARG for an unknown option, HO_ERR_RANGE for a value out of range. */
#define HO_OPT_GRAPH 1
#define HO_OPT_ROUNDS 2
#define HO_OPT_ROUND_CHUNK 3
#define HO_OPT_FP64_CHECK 4
#define HO_OPT_TIME_ROUNDS 5
#define HO_OPT_TENSOR 6
#define HO_OPT_TAIL 7
#define HO_OPT_GPU_FIT 8
#define HO_OPT_LAST_FIT_GPU 9
#define HO_OPT_WARM_CAP 10
int ho_set_option(ho_context* ctx, int option, int64_t value);
/* Path tracing with Lambertian bounces (replaces: render_kernel at spp
 * samples and depth max_depth, FEM-AABB/raytracer.cu:410-476, with
 * ray_color :362-406 and scatter :60-98). Per pixel and sample one path
 * through a jittered point of the pixel; each intersection multiplies the
 * path's attenuation by the albedo (boundary face 0 of a hex 0.1/0.2/0.8,
 * every other hit 0.5 grey, as main.cu:39-41 and raytracer.cu:248 assign);
 * a miss adds attenuation x sky; a path still going after max_depth
 * intersections adds black. Image = gamma-2 average over the samples, 8 bits,
 * rows as ho_render, one image per isovalue. Random numbers are hashed from
 * (seed, path, bounce), so an image is reproducible for a given seed (the
 * reference seeds curand with the time). Every bounce is one call of the
 * intersection engine in the context's solver mode. rays_traced (may be
 * NULL): ray queries over all bounces. W * H * spp must stay below 2^32. */
int ho_path_trace(ho_context* ctx, const ho_camera* cam, const float* isovalues, int n_iso, int W, int H, int spp,
                  int max_depth, uint64_t seed, int iso_zero_disables, uint8_t* rgb_out, int64_t* rays_traced);
/* Device-buffer form; synchronises the stream once per bounce (it reads the
 * number of paths still alive). */
int ho_path_trace_device(ho_context* ctx, const ho_camera* cam, const float* isovalues, int n_iso, int W, int H,
                         int spp, int max_depth, uint64_t seed, int iso_zero_disables, uint8_t* rgb_dev,
                         int64_t* rays_traced, void* stream);

/* The FP64 residuals that the batched / learned engines' final check
 * computes, for caller-given hits (no reference counterpart): for hit i on
 * ray i (rays as in ho_intersect), out[2i] = the largest component of
 * |x(xi) - (o + t d)| and out[2i+1] = the field value u(xi) (0 for misses and
 * elements without field). HO_ERR_RANGE when a hit names no element. */
int ho_hit_residuals(ho_context* ctx, int64_t n, const float* rays, const ho_hit* hits, double* out);
int ho_get_option(ho_context* ctx, int option, int64_t* value);

/* Autotuner of the batched / learned engine (no reference counterpart): times
 * the given render (device buffers only, CUDA events on the context's stream,
 * one warm-up and one timed call per candidate) for HO_AUTOTUNE_N element
 * batch sizes (0.5, 1, 2, 4 and 8 times the kernel's pair slots), keeps the
 * fastest as HO_OPT_ROUND_CHUNK and returns it in *chunk_out; ms_out (may be
 * NULL) receives the candidates' times. Uses the current mode. */
#define HO_AUTOTUNE_N 5
int ho_autotune(ho_context* ctx, const ho_camera* cam, const float* isovalues, int n_iso, int width, int height,
                int iso_zero_disables, int64_t* chunk_out, int64_t* candidates_out, float* ms_out);

/* ---- learned mode (no reference counterpart) ------------------------------
 * Network 48 -> 128 -> 128 -> 128 -> 8 (GELU), BF16 weights, FP32
 * accumulation. Flat parameter order: W1[48][128], b1[128], W2[128][128], b2,
 * W3[128][128], b3, W4[128][8], b4[8] (HO_MLP_PARAMS floats; W[in][out]).
 * Input of one (ray, element) pair: element descriptor (8 corners and 6
 * face-centre offsets in the element frame, 42) + entry point into the
 * element's padded box in that frame (3) + unit direction (3). Outputs:
 * reference coordinates at the entry (3), their rate of change along the ray
 * per element size (3), 2 unused. */
#define HO_MLP_PARAMS 40328
#define HO_MLP_IN 48
#define HO_MLP_OUT 8
int ho_mlp_init(ho_context* ctx, uint64_t seed);
int ho_mlp_set_params(ho_context* ctx, const float* params);
int ho_mlp_get_params(ho_context* ctx, float* params);
/* Y[n][8] = network(X[n][48]) with the inference kernel. */
int ho_mlp_forward(ho_context* ctx, const float* X, int64_t n, float* Y);
/* One forward/backward pass of the training kernels on n rows: masked MSE on
 * outputs 0..5 (mean over valid rows); gradients in the flat order. */
int ho_mlp_grad(ho_context* ctx, const float* X, const float* T, const uint8_t* valid, int n, float* loss,
                float* grads);
/* n training pairs produced by the plain solver on seeded random rays through
 * random elements of the built scene: X[n][48], T[n][8], valid[n]. */
int ho_learn_samples(ho_context* ctx, int64_t n, uint64_t seed, float* X, float* T, uint8_t* valid);
/* Generate n_samples pairs on the device and train (Adam, cosine decay);
 * losses (optional) receives the per-step batch loss. */
int ho_train_mlp(ho_context* ctx, int64_t n_samples, int steps, int batch, float lr, uint64_t seed, float* losses);
/* Checkpoint: FP32 master parameters + their BF16 copy. */
int ho_mlp_save(ho_context* ctx, const char* path);
int ho_mlp_load(ho_context* ctx, const char* path);
/* Counters of the last trace call. After a *_device call on a caller's stream
 * it waits for that call's work on that stream first (an event recorded at
 * the end of the call); a call enqueued while its stream was being captured
 * records no event, and its counters appear once the graph has run and a
 * later call or read finds them. */
int ho_get_stats(ho_context* ctx, ho_stats* out);

/* FP32 FMA throughput of the device in TFLOP/s (register-resident FMA loop):
 * the roofline denominator for the CUDA-core-bound intersection kernels. No
 * reference counterpart. */
int ho_measure_fp32_peak(int device, double* tflops);

/* Replaces: save_image_ppm (FEM-AABB/raytracer.cu:480-494). P6, rows in
 * buffer order. */
int ho_save_ppm(const uint8_t* rgb, int width, int height, const char* path);
/* Beside save_image_ppm (FEM-AABB/raytracer.cu:480-494), which is the
 * reference's only image writer: the same image as an 8-bit RGB PNG, rows in
 * buffer order, uncompressed (stored deflate blocks). HO_ERR_ARG on a NULL
 * argument or a size <= 0; HO_ERR_RANGE when the image data would exceed
 * 2^31 bytes; HO_ERR_IO when the file cannot be written. */
int ho_save_png(const uint8_t* rgb, int width, int height, const char* path);

#ifdef __cplusplus
}
#endif
#endif /* HORENDER_H */
