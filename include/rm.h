/*
 * rm.h -- C ABI of the GB300 renderer hot path (radii, culling, marcher,
 * batched marcher, backward).
 *
 * The reference exposes this path as two in-process C++ classes, not as an
 * FFI: kdtree::KDTreeFlann (src/kdtree/kdtree_flann.h:15-43: Build, Search
 * with KDTreeSearchParams{knn}) and the PointcloudRayMarcher singleton
 * (src/ray_marching.h:11-44: get_instance(vertices, colors, radii, tree),
 * render_to_texture(cam2world, fov, texture)).  This header replaces both
 * with plain C entry points: plain pointers and sizes, one explicit CUDA
 * stream per context, status codes instead of exit(1)
 * (src/utils.h:29-45), and no process-wide singleton (the reference keeps
 * its state in __device__ globals, src/ray_marching.cu:17-38).
 *
 * Conventions
 *   - Every function returns rm_status; on failure rm_last_error(ctx)
 *     returns a message.  Nothing calls exit().
 *   - A context owns all device memory it allocates; caller pointers are
 *     borrowed for the duration of a call only.
 *   - `loc` says where caller buffers live: RM_HOST (pageable or pinned host
 *     memory; the call synchronises before it returns) or RM_DEVICE (device
 *     pointers on the context's device; the call is asynchronous on the
 *     context's stream, use rm_synchronize).  Render outputs in pinned host
 *     memory are written by the kernel directly; pageable ones are staged on
 *     the device and copied after the kernel.
 *   - One context per host thread.  Contexts are independent.
 *   - Images are row-major W x H with row 0 at the BOTTOM (the reference
 *     renders into an OpenGL texture whose row 0 is the bottom row); the
 *     file writers flip them, as the reference does (src/utils.cu:161, 172-178).
 *   - Point indices are positions in the caller's (PLY) order.
 */
#ifndef RM_H
#define RM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  RM_OK = 0,
  RM_ERR_INVALID = 1,   /* bad argument */
  RM_ERR_STATE = 2,     /* call out of order (e.g. render before radii) */
  RM_ERR_CUDA = 3,      /* CUDA runtime error */
  RM_ERR_OOM = 4,       /* device allocation failed */
  RM_ERR_LIMIT = 5,     /* a size above a documented maximum */
  RM_ERR_KERNEL = 6     /* a kernel reported an internal error flag */
} rm_status;

enum { RM_HOST = 0, RM_DEVICE = 1 };

typedef struct rm_ctx rm_ctx;

/* Constants of the reference (src/common.h:4-11, src/ray_marching.h:17)
 * plus the GB300 launch knobs.  rm_config_default fills the reference's
 * values; the marcher's constants are compile-time in the reference and
 * are kept fixed here (other values are rejected) so results stay equal. */
typedef struct {
  float zfar;            /* 100.0 (ZFAR) */
  float znear;           /* 0.1 (ZNEAR) */
  int32_t max_steps;     /* 128 (MAX_STEPS) */
  float min_dist;        /* 1e-3 (MIN_DIST) */
  int32_t knn;           /* 10 (PointcloudRayMarcher::knn) */
  int32_t leaf_size;     /* points per index leaf: 8, 16 or 32 (default 16) */
  int32_t device;        /* CUDA device ordinal (default 0) */
  void* stream;          /* cudaStream_t to use; NULL: the context creates one */
} rm_config;

/* One camera (render_to_texture's arguments, src/ray_marching.cu:93-96). */
typedef struct {
  float cam2world[16];   /* column-major 4x4, OpenGL camera (-Z forward, +Y up) */
  int32_t width;         /* pixels; the reference uses (int)(2 * cx) */
  int32_t height;        /* pixels; (int)(2 * cy) */
  float fov;             /* horizontal field of view, radians (main.cu:206) */
} rm_view;

/* Per-view outputs; any pointer may be NULL. W*H elements each. */
typedef struct {
  float* rgbd;           /* float4 per pixel: colour rgb and depth in .w, as
                            the reference's RGBA32F texture; (0,0,0,0) on a miss */
  int32_t* hit;          /* first-hit point index, -1 on a miss */
  float* depth;          /* depth along the ray, 0 on a miss */
  int32_t* steps;        /* distance-function evaluations per ray */
} rm_frame;

/* Launch statistics of the last render call. */
typedef struct {
  int64_t rays;          /* rays marched */
  int64_t steps;         /* total distance-function evaluations */
  int64_t hits;          /* rays that hit a sphere */
  int64_t packet_steps;  /* steps answered by a warp packet traversal */
  int64_t solo_steps;    /* steps answered by a per-ray tree walk */
  int64_t packet_leaves; /* leaves scanned by packet traversals */
  int64_t packet_nodes;  /* tree nodes expanded by packet traversals */
  int64_t warp_steps;    /* warp-wide distance steps */
  int64_t split_steps;   /* warp steps whose lanes were split into two packets (the best-first
                            walk does not split; kept for layout, always 0) */
  int64_t search_errors; /* searches that hit a self-check bound (0 unless the index is broken) */
  float kernel_ms;       /* device time of the last render launch (graph for the batch) */
  int64_t queue_spills;  /* best-first walk: pending nodes moved from the 32-entry register queue
                            to the warp's shared-memory overflow stack */
  int64_t dfs_walks;     /* best-first walks whose overflow stack filled too, so that they
                            finished in depth-first order (exact either way) */
} rm_stats;

/* Marcher launch parameters (picked by rm_autotune or set by hand). */
typedef struct {
  int32_t tile_w;        /* warp tile width in pixels (tile_w * tile_h == 32) */
  int32_t tile_h;
  int32_t rays_per_lane; /* tiles per work item; a lane whose ray ends takes the item's next pixel */
  int32_t ctas_per_sm;   /* resident 4-warp CTAs per SM (1-16; the packet marchers have register-
                            capped instances for 4-8: 128, 96, 80, 72 or 64 registers per
                            thread; default 8) */
  int32_t search;        /* 1: the warp walks the index once for all its rays (packet
                            traversal, default); 0: every ray walks it alone */
} rm_launch;

void rm_config_default(rm_config* cfg);

/* Replaces PointcloudRayMarcher::get_instance (src/ray_marching.cu:159-168)
 * and the device-side set-up of its constructor (:170-200). */
rm_status rm_ctx_create(const rm_config* cfg, rm_ctx** out);
void rm_ctx_destroy(rm_ctx* ctx);
const char* rm_last_error(const rm_ctx* ctx);
rm_status rm_synchronize(rm_ctx* ctx);

/* Upload the cloud (main.cu:73-92: PLY vertices as xyz, colours as uint8
 * RGB divided by 255).  xyz has `stride` floats per point (>= 3); rgb is
 * 3 bytes per point or NULL (white).  Copies into context-owned storage. */
rm_status rm_cloud_set(rm_ctx* ctx, const float* xyz, int32_t stride, const uint8_t* rgb,
                       int64_t n, int32_t loc);

/* Build the spatial index (replaces KDTreeFlann::Build,
 * src/kdtree/kdtree_flann.cu:101-117 -> CudaKdTreeBuilder::buildTree,
 * kdtree_cuda_builder.h:483-599): Morton keys, radix sort, packed float4
 * records, implicit 4-ary box tree.  Fully on the device. */
rm_status rm_index_build(rm_ctx* ctx);

/* Exact k nearest neighbours (k <= 32) of m query points (xyz, stride
 * floats each), ordered by (squared distance, index); replaces
 * KDTreeFlann::SearchKNN (src/kdtree/kdtree_flann.cu:65-80).  Rows are
 * padded with index -1 / +inf when the cloud has fewer than k points. */
rm_status rm_knn(rm_ctx* ctx, const float* queries, int32_t stride, int64_t m, int32_t k,
                 int32_t* idx_out, float* d2_out, int32_t loc);

/* Radii precompute (main.cu:107-113): for every point, sqrt of the squared
 * distance of the second entry of its self-inclusive 2-NN list.
 * radii_out (may be NULL) receives the unclamped values (what the
 * .kdtree.radii cache stores); nn_out (may be NULL) that entry's index.
 * The context keeps min(r, max_radius) for rendering when max_radius > 0
 * (main.cu:144-149). */
rm_status rm_radii_compute(rm_ctx* ctx, float max_radius, float* radii_out, int32_t* nn_out,
                           int32_t loc);

/* Use cached radii (main.cu:122-141), n values in cloud order, clamped as
 * above. */
rm_status rm_radii_set(rm_ctx* ctx, const float* radii, int64_t n, float max_radius,
                       int32_t loc);

/* Pane distance W / (2 tanf(fov / 2)) of each view as the render kernel
 * evaluates it on the device (src/ray_marching.cu:74). */
rm_status rm_view_pane(rm_ctx* ctx, const rm_view* views, int32_t n, float* pane_out);

/* Plain form: one view per launch (replaces render_to_texture +
 * render<<<>>>, src/ray_marching.cu:63-154; the GL texture becomes `out`). */
rm_status rm_render(rm_ctx* ctx, const rm_view* view, const rm_frame* out, int32_t loc);

/* Batched form: all views in one persistent launch over a shared work queue
 * of ray tiles, replayed as a CUDA graph.  Results equal rm_render's. */
rm_status rm_render_batch(rm_ctx* ctx, const rm_view* views, int32_t n, const rm_frame* out,
                          int32_t loc);

rm_status rm_set_launch(rm_ctx* ctx, const rm_launch* launch);
rm_status rm_get_launch(rm_ctx* ctx, rm_launch* launch);

/* Autotuner: times candidate tile shapes, CTAs per SM, search modes (with
 * rays per lane for the per-ray walk) and index leaf sizes on the given
 * views (device-resident scratch outputs) and keeps the fastest.  Rebuilds
 * the index when the leaf size changes.  `best_ms` (may be NULL) receives
 * the winning time. */
rm_status rm_autotune(rm_ctx* ctx, const rm_view* views, int32_t n, rm_launch* chosen,
                      int32_t* leaf_size, float* best_ms);

rm_status rm_get_stats(rm_ctx* ctx, rm_stats* stats);

/* Backward (no reference counterpart: the reference has no gradient path).
 * For each view and pixel with hit[p] >= 0, accumulates
 *   g_rgb[hit]    += dl_drgb[p]                      (3 floats per pixel)
 *   g_xyz[hit]    += dl_ddepth[p] * d t / d centre   (3 floats per point)
 *   g_radius[hit] += dl_ddepth[p] * d t / d radius
 * where t is the entry distance of the pixel's ray into the sphere of its
 * stored hit point (closest-approach distance when the ray misses that
 * sphere, with zero radius gradient).  hit comes from the forward pass, so
 * no marching trace is stored.  Gradient arrays are in cloud order, are
 * accumulated into (zero them first) and must be device pointers when
 * loc == RM_DEVICE.  Per view v the pixel arrays start at offsets
 * sum_{u<v} W_u*H_u. */
rm_status rm_backward(rm_ctx* ctx, const rm_view* views, int32_t n, const float* dl_drgb,
                      const float* dl_ddepth, const int32_t* hit, float* g_rgb, float* g_xyz,
                      float* g_radius, int32_t loc);

/* Number of points in the context's cloud. */
int64_t rm_cloud_size(const rm_ctx* ctx);

/* Allocation-free batched form (no counterpart in the reference).  For
 * callers that cannot allocate device memory: an application whose GPU
 * memory is all handed out by its own pool, a process under a fixed device
 * memory cap, or a loop that cannot afford the device-wide synchronisation
 * of cudaMalloc/cudaFree.  Renders like rm_render_batch into DEVICE outputs
 * (every non-NULL rm_frame pointer is a device pointer), but allocates
 * nothing and uses no CUDA graph: its scratch (work queue, counters and a
 * view table) is one static device array of RM_NOALLOC_SCRATCH_BYTES that
 * every GPU loading the library holds until exit.  At most
 * RM_NOALLOC_MAX_VIEWS views per call (more returns RM_ERR_LIMIT); the cloud
 * must be non-empty.  The first call on a device looks up the array's device
 * address; make it before any stream capture.  That address is kept for the
 * process's life: it belongs to the device's primary context (the CUDA
 * runtime's own), and a cudaDeviceReset after the first call invalidates it.
 * All calls share the array: calls that overlap on the GPU race, so
 * serialise them.  Returns after the frames are written (it synchronises the
 * context's stream).  rm_get_stats does not count its work: after this call
 * it reports zeros until the next rm_render or rm_render_batch. */
#define RM_NOALLOC_MAX_VIEWS 1024
#define RM_NOALLOC_SCRATCH_BYTES (256 + 1024 * 136)
rm_status rm_render_batch_noalloc(rm_ctx* ctx, const rm_view* views, int32_t n,
                                  const rm_frame* out);

#ifdef __cplusplus
}
#endif
#endif /* RM_H */
