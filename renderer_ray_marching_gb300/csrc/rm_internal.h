// rm_internal.h -- host-side context of the C ABI and the launch entry
// points shared between translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "rm.h"
#include "rm_device.cuh"

namespace rm {

// Thrown by CK on a CUDA error; the API layer turns it into RM_ERR_CUDA.
struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct OomError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define CK(expr)                                                                         \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess)                                                               \
      throw ::rm::CudaError(std::string(#expr) + ": " + cudaGetErrorString(_e));          \
  } while (0)

// Grow-only device buffer owned by a context.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  void reserve(size_t bytes) {
    if (bytes <= cap) return;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      throw OomError("cudaMalloc of " + std::to_string(want) + " bytes failed: " +
                     cudaGetErrorString(e));
    }
    cap = want;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* ptr() const {
    return reinterpret_cast<T*>(p);
  }
};

// Per-view record read by the batched kernel (one per view of a batch).
struct ViewDev {
  float m[16];          // column-major cam-to-world
  int32_t width, height;
  float fov;
  float pane;           // resolved on the device
  int32_t tiles_x;      // warp tiles across
  int32_t tiles_y;
  int64_t tile_base;    // first work item of this view
  float reserved[2];    // keeps the 136-byte layout the allocation-free scratch is sized for
  float4* rgbd;
  int32_t* hit;
  float* depth;
  int32_t* steps;
};

struct Ctx {
  rm_config cfg{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  int sm_count = 0;

  int64_t n = 0;
  bool have_cloud = false, have_index = false, have_radii = false;
  float bounds[6] = {0, 0, 0, 0, 0, 0};
  float max_r = INFINITY;  // largest clamped radius (host copy, for culling)
  int depth = 0;
  int64_t nleaves = 0;

  DevBuf pos;            // float4 cloud order (x, y, z, 0)
  DevBuf rgb;            // uint32 packed rgb, cloud order
  DevBuf radii_clamped;  // float cloud order (what rendering uses)
  DevBuf rec, col;       // float4 sorted
  DevBuf perm, iperm;    // int32
  DevBuf groups;         // float4 child groups
  DevBuf keys[2], vals[2];
  DevBuf sort_counts, scan_sums, scratch_bounds;
  DevBuf scalars;        // [0..6] bounds + flag, [8] max radius bits, [16..] counters
  DevBuf staging_in, staging_out;
  DevBuf views;          // ViewDev table
  DevBuf frame_bufs;     // device outputs for host-side frames
  DevBuf queue;          // work-queue counters

  rm_launch launch{8, 4, 1, 8, 1};
  rm_stats stats{};
  // set by the allocation-free batch, whose counters live in its static
  // scratch: rm_get_stats then reports zeros instead of the counters and
  // time of an earlier render
  bool stats_from_noalloc = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // cached CUDA graph of the batched launch
  cudaGraphExec_t graph_exec = nullptr;
  void* graph_key_views = nullptr;
  int graph_key_n = -1;
  rm_launch graph_key_launch{0, 0, 0, 0, 0};
  void* pinned_views = nullptr;
  size_t pinned_views_cap = 0;

  IndexDev index() const {
    IndexDev ix;
    ix.rec = rec.ptr<float4>();
    ix.col = col.ptr<float4>();
    ix.groups = groups.ptr<float4>();
    ix.perm = perm.ptr<int32_t>();
    ix.n = n;
    ix.leaf = cfg.leaf_size;
    ix.depth = depth;
    return ix;
  }
  void drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    graph_key_n = -1;
  }
};

// rm_index.cu
void launch_pack_points(Ctx& c, const float* xyz, int stride, int64_t n);
void launch_pack_colours(Ctx& c, const uint8_t* rgb, int64_t n);
void launch_clamp_radii(Ctx& c, const float* in, float max_radius);
void launch_clamp_radii_only(Ctx& c, const float* in, float max_radius);
void launch_set_radius(Ctx& c);
void refresh_max_radius(Ctx& c);
bool build_index(Ctx& c);

// rm_radii.cu
void launch_radii(Ctx& c, float max_radius, float* radii_out, int32_t* nn_out);
void launch_knn(Ctx& c, const float* q, int stride, int64_t m, int k, int32_t* idx, float* d2);

// rm_march.cu
void launch_view_pane(Ctx& c, const rm_view* views_dev, int n, float* pane_out);
void launch_render_plain(Ctx& c, const rm_view& v, float4* rgbd, int32_t* hit, float* depth,
                         int32_t* steps, unsigned long long* counters);
void launch_render_batch(Ctx& c, ViewDev* views_dev, int n, int64_t total_items,
                         const rm_launch& L, unsigned long long* queue, unsigned long long* counters);
void launch_prepare_views(Ctx& c, ViewDev* views_dev, int n, unsigned long long* counters);

// rm_backward.cu
void launch_backward(Ctx& c, const ViewDev* views_dev, int n, int64_t total_pixels,
                     const int64_t* pix_base, const float* dl_drgb, const float* dl_ddepth,
                     const int32_t* hit, float* g_rgb, float* g_xyz, float* g_radius);

}  // namespace rm

struct rm_ctx {
  rm::Ctx c;
};
