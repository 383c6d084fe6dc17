// rm_noalloc.cu -- rm_render_batch_noalloc: the batched marcher for callers
// that cannot allocate device memory.
//
// Who cannot allocate: a host application whose device memory is handed out
// entirely by its own pool (a caching allocator such as PyTorch's, or an
// engine that reserves the GPU at start-up), a process under a fixed device
// memory cap, and a render loop that must not pay for the implicit
// device-wide synchronisation of cudaMalloc/cudaFree or cudaMallocHost.
// rm_render_batch grows a context-owned view table, a pinned host table and
// staging frames on demand; this entry point does none of that.
//
// Its scratch -- the work-queue counter, the statistics counters and the
// per-view table the persistent kernel reads -- is one file-scope
// __device__ array of RM_NOALLOC_SCRATCH_BYTES (136.25 KB), which every GPU
// that loads the library holds until the process exits.  All calls, from
// every context on a device, share it and it keeps the last call's contents:
// the queue and the counters are cleared at the start of every call, and the
// view table is rewritten.  Calls that overlap on the GPU (two streams, two
// contexts on one device, two host threads) race on it; serialise them.
//
// In host code the array's name is only a host-side stand-in for the symbol,
// not a device address.  The device address comes from cudaGetSymbolAddress,
// taken once per device, with that device current, by the first call made
// on it; make that first call before any stream capture begins.  The address
// is kept for the life of the process, so it belongs to the device's primary
// context (the one the CUDA runtime uses): after a cudaDeviceReset it is no
// longer valid (neither is any rm_ctx created before the reset).
#include "rm_internal.h"

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

namespace rm {
namespace {

constexpr size_t kHeaderBytes = 256;  // [0] queue counter, [16..31] counters
constexpr size_t kScratchBytes = kHeaderBytes + (size_t)RM_NOALLOC_MAX_VIEWS * sizeof(ViewDev);
static_assert(kScratchBytes == RM_NOALLOC_SCRATCH_BYTES, "RM_NOALLOC_SCRATCH_BYTES does not match the layout");

static __device__ __align__(256) unsigned char g_scratch[RM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;                          // guards g_scratch_dev and g_host_views
void* g_scratch_dev[kMaxDevices] = {};    // device address of g_scratch, per device
ViewDev g_host_views[RM_NOALLOC_MAX_VIEWS];  // host copy of the view table

rm_status fail(Ctx& c, rm_status s, const char* what) {
  c.err = std::string("rm_render_batch_noalloc: ") + what;
  return s;
}

bool view_valid(const rm_view& v) {
  if (v.width <= 0 || v.height <= 0 || (int64_t)v.width * v.height > (1ll << 31) - 1) return false;
  if (!std::isfinite(v.fov) || v.fov <= 0.0f) return false;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(v.cam2world[i])) return false;
  return true;
}

}  // namespace
}  // namespace rm

using namespace rm;

extern "C" rm_status rm_render_batch_noalloc(rm_ctx* ctx, const rm_view* views, int32_t n,
                                             const rm_frame* out) {
  if (!ctx) return RM_ERR_INVALID;
  Ctx& c = ctx->c;
  c.err.clear();
  if (n < 0 || (n > 0 && (!views || !out))) return fail(c, RM_ERR_INVALID, "bad arguments");
  if (n > RM_NOALLOC_MAX_VIEWS) return fail(c, RM_ERR_LIMIT, "more views than RM_NOALLOC_MAX_VIEWS (1024)");
  if (!c.have_index || !c.have_radii) return fail(c, RM_ERR_STATE, "index and radii must be ready");
  if (c.n == 0) return fail(c, RM_ERR_STATE, "the cloud is empty");
  if (n == 0) return RM_OK;
  for (int v = 0; v < n; ++v)
    if (!view_valid(views[v]))
      return fail(c, RM_ERR_INVALID, "a view has a bad size, fov or matrix");
  if (c.cfg.device < 0 || c.cfg.device >= kMaxDevices) return fail(c, RM_ERR_INVALID, "device index out of range");

  std::lock_guard<std::mutex> lock(g_mu);
  cudaError_t e = cudaSetDevice(c.cfg.device);
  if (e != cudaSuccess) return fail(c, RM_ERR_CUDA, cudaGetErrorString(e));
  if (!g_scratch_dev[c.cfg.device]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return fail(c, RM_ERR_CUDA, cudaGetErrorString(e));
    g_scratch_dev[c.cfg.device] = p;
  }
  unsigned char* base = static_cast<unsigned char*>(g_scratch_dev[c.cfg.device]);
  unsigned long long* queue = reinterpret_cast<unsigned long long*>(base);
  unsigned long long* counters = queue + 16;
  ViewDev* views_dev = reinterpret_cast<ViewDev*>(base + kHeaderBytes);

  const rm_launch L = c.launch;
  c.stats_from_noalloc = true;  // its counters stay in the static scratch
  int64_t items = 0;
  for (int v = 0; v < n; ++v) {
    ViewDev& d = g_host_views[v];
    memset(&d, 0, sizeof(d));
    memcpy(d.m, views[v].cam2world, sizeof(d.m));
    d.width = views[v].width;
    d.height = views[v].height;
    d.fov = views[v].fov;
    d.tiles_x = (d.width + L.tile_w - 1) / L.tile_w;
    const int ih = L.tile_h * L.rays_per_lane;
    d.tiles_y = (d.height + ih - 1) / ih;
    d.tile_base = items;
    items += (int64_t)d.tiles_x * d.tiles_y;
    d.rgbd = reinterpret_cast<float4*>(out[v].rgbd);
    d.hit = out[v].hit;
    d.depth = out[v].depth;
    d.steps = out[v].steps;
  }
  // The source is pageable, so the copy has taken g_host_views when it returns.
  e = cudaMemcpyAsync(views_dev, g_host_views, (size_t)n * sizeof(ViewDev), cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(base, 0, kHeaderBytes, c.stream);
  if (e != cudaSuccess) return fail(c, RM_ERR_CUDA, cudaGetErrorString(e));
  launch_prepare_views(c, views_dev, n, counters);
  launch_render_batch(c, views_dev, n, items, L, queue, counters);
  e = cudaGetLastError();
  unsigned long long bad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, counters + 3, sizeof(bad), cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return fail(c, RM_ERR_CUDA, cudaGetErrorString(e));
  if (bad) return fail(c, RM_ERR_KERNEL, "a nearest-neighbour search did not complete");
  return RM_OK;
}
