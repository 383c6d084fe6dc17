// rm_api.cu -- the extern "C" entry points declared in include/rm.h.
//
// Every entry point catches all exceptions and converts them into an
// rm_status with the message kept in the context (the reference instead
// prints and calls exit(1), src/utils.h:29-45).
#include "rm_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

using namespace rm;

namespace {

constexpr int kCounters = 16;  // unsigned long long slots at scalars + 16

unsigned long long* counters(Ctx& c) { return c.scalars.ptr<unsigned long long>() + 16; }
unsigned long long* err_counter(Ctx& c) { return c.scalars.ptr<unsigned long long>() + 8; }

rm_status fail(Ctx& c, rm_status s, const std::string& msg) {
  c.err = msg;
  return s;
}

struct KernelError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

template <class F>
rm_status guarded(rm_ctx* ctx, F&& f) {
  if (!ctx) return RM_ERR_INVALID;
  Ctx& c = ctx->c;
  try {
    if (c.cfg.device >= 0) CK(cudaSetDevice(c.cfg.device));
    c.err.clear();
    return f(c);
  } catch (const KernelError& e) {
    c.err = e.what();
    return RM_ERR_KERNEL;
  } catch (const OomError& e) {
    c.err = e.what();
    return RM_ERR_OOM;
  } catch (const CudaError& e) {
    c.err = e.what();
    return RM_ERR_CUDA;
  } catch (const std::bad_alloc&) {
    c.err = "host allocation failed";
    return RM_ERR_OOM;
  } catch (const std::exception& e) {
    c.err = e.what();
    return RM_ERR_CUDA;
  }
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Device pointer for a caller buffer of `bytes`: the pointer itself for
// RM_DEVICE, else a staging buffer (filled from host when `upload`).
const void* stage_in(Ctx& c, DevBuf& buf, const void* src, size_t bytes, int loc) {
  if (!src) return nullptr;
  if (loc == RM_DEVICE) return src;
  buf.reserve(bytes);
  CK(cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, c.stream));
  return buf.p;
}

// Error slots: the radii/kNN kernels count failed searches at err_counter,
// the marchers at counters[3] (stack bound or node budget exceeded).
void check_kernel_errors(Ctx& c) {
  unsigned long long e[2] = {0, 0};
  CK(cudaMemcpyAsync(&e[0], err_counter(c), sizeof(e[0]), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(&e[1], counters(c) + 3, sizeof(e[1]), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (e[0] || e[1])
    throw KernelError("kernel reported " + std::to_string(e[0] + e[1]) + " incomplete nearest-neighbour searches");
}

bool view_ok(const rm_view& v, std::string* why) {
  if (v.width <= 0 || v.height <= 0) {
    *why = "view width and height must be positive";
    return false;
  }
  if ((int64_t)v.width * v.height > (1ll << 31) - 1) {
    *why = "view has more than 2^31-1 pixels";
    return false;
  }
  if (!std::isfinite(v.fov) || v.fov <= 0.0f) {
    *why = "view fov must be finite and positive";
    return false;
  }
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(v.cam2world[i])) {
      *why = "view matrix has non-finite entries";
      return false;
    }
  return true;
}

struct FrameStaging {
  float4* rgbd;
  int32_t* hit;
  float* depth;
  int32_t* steps;
};

// Device-visible address of a caller's host buffer when it is pinned
// (page-locked and mapped into the device's address space), else nullptr.
// The marchers write such buffers directly over the CPU-GPU link while they
// run, so a host-side frame costs no staging buffer and no copy phase after
// the kernel; pageable buffers keep the stage-then-copy path.
void* pinned_device_ptr(void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return at.devicePointer;
}

// Every non-NULL output of `out` pinned?  Then `f` gets their device-visible
// addresses.
bool frame_pinned(const rm_frame& out, FrameStaging* f) {
  FrameStaging g{nullptr, nullptr, nullptr, nullptr};
  if (out.rgbd && !(g.rgbd = (float4*)pinned_device_ptr(out.rgbd))) return false;
  if (out.hit && !(g.hit = (int32_t*)pinned_device_ptr(out.hit))) return false;
  if (out.depth && !(g.depth = (float*)pinned_device_ptr(out.depth))) return false;
  if (out.steps && !(g.steps = (int32_t*)pinned_device_ptr(out.steps))) return false;
  *f = g;
  return true;
}

}  // namespace

extern "C" {

void rm_config_default(rm_config* cfg) {
  if (!cfg) return;
  cfg->zfar = ZFAR;
  cfg->znear = ZNEAR;
  cfg->max_steps = MAX_STEPS;
  cfg->min_dist = MIN_DIST;
  cfg->knn = KNN;
  cfg->leaf_size = 16;
  cfg->device = 0;
  cfg->stream = nullptr;
}

rm_status rm_ctx_create(const rm_config* cfg, rm_ctx** out) {
  if (!out) return RM_ERR_INVALID;
  *out = nullptr;
  rm_config def;
  rm_config_default(&def);
  const rm_config& k = cfg ? *cfg : def;
  if (k.zfar != ZFAR || k.znear != ZNEAR || k.max_steps != MAX_STEPS || k.min_dist != MIN_DIST ||
      k.knn != KNN)
    return RM_ERR_INVALID;  // the reference's marcher constants are fixed
  if (k.leaf_size != 8 && k.leaf_size != 16 && k.leaf_size != 32) return RM_ERR_INVALID;
  rm_ctx* ctx = new (std::nothrow) rm_ctx();
  if (!ctx) return RM_ERR_OOM;
  ctx->c.cfg = k;
  rm_status s = guarded(ctx, [&](Ctx& c) -> rm_status {
    int dev = c.cfg.device;
    CK(cudaSetDevice(dev));
    CK(cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, dev));
    if (c.cfg.stream) {
      c.stream = (cudaStream_t)c.cfg.stream;
    } else {
      CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
      c.own_stream = true;
    }
    c.scalars.reserve(1024);
    CK(cudaMemsetAsync(c.scalars.p, 0, 1024, c.stream));
    c.queue.reserve(256);
    CK(cudaEventCreate(&c.ev0));
    CK(cudaEventCreate(&c.ev1));
    CK(cudaStreamSynchronize(c.stream));
    return RM_OK;
  });
  if (s != RM_OK) {
    rm_ctx_destroy(ctx);
    return s;
  }
  *out = ctx;
  return RM_OK;
}

void rm_ctx_destroy(rm_ctx* ctx) {
  if (!ctx) return;
  Ctx& c = ctx->c;
  cudaSetDevice(c.cfg.device);
  if (c.stream) cudaStreamSynchronize(c.stream);
  c.drop_graph();
  DevBuf* bufs[] = {&c.pos, &c.rgb, &c.radii_clamped, &c.rec, &c.col, &c.perm, &c.iperm,
                    &c.groups, &c.keys[0], &c.keys[1], &c.vals[0], &c.vals[1], &c.sort_counts,
                    &c.scan_sums, &c.scratch_bounds, &c.scalars, &c.staging_in, &c.staging_out,
                    &c.views, &c.frame_bufs, &c.queue};
  for (DevBuf* b : bufs) b->release();
  if (c.pinned_views) cudaFreeHost(c.pinned_views);
  if (c.ev0) cudaEventDestroy(c.ev0);
  if (c.ev1) cudaEventDestroy(c.ev1);
  if (c.own_stream && c.stream) cudaStreamDestroy(c.stream);
  delete ctx;
}

const char* rm_last_error(const rm_ctx* ctx) {
  if (!ctx) return "null context";
  return ctx->c.err.c_str();
}

rm_status rm_synchronize(rm_ctx* ctx) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    CK(cudaStreamSynchronize(c.stream));
    return RM_OK;
  });
}

int64_t rm_cloud_size(const rm_ctx* ctx) { return ctx ? ctx->c.n : -1; }

rm_status rm_cloud_set(rm_ctx* ctx, const float* xyz, int32_t stride, const uint8_t* rgb, int64_t n,
                       int32_t loc) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (n < 0 || (n > 0 && !xyz) || stride < 3 || (loc != RM_HOST && loc != RM_DEVICE))
      return fail(c, RM_ERR_INVALID, "rm_cloud_set: bad arguments");
    if (n > (1ll << 31) - 2) return fail(c, RM_ERR_LIMIT, "rm_cloud_set: more than 2^31-2 points");
    c.drop_graph();
    c.have_cloud = c.have_index = c.have_radii = false;
    c.n = n;
    c.max_r = INFINITY;
    size_t np = (size_t)(n > 0 ? n : 1);
    c.pos.reserve(np * sizeof(float4));
    c.rgb.reserve(np * sizeof(uint32_t));
    if (n > 0) {
      const float* dx = (const float*)stage_in(c, c.staging_in, xyz, (size_t)n * stride * sizeof(float), loc);
      launch_pack_points(c, dx, stride, n);
      const uint8_t* dr = nullptr;
      if (rgb) {
        // staging_in may still be read by the pack kernel: use staging_out for colours
        dr = (const uint8_t*)stage_in(c, c.staging_out, rgb, (size_t)n * 3, loc);
      }
      launch_pack_colours(c, dr, n);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(c.stream));
    }
    c.have_cloud = true;
    return RM_OK;
  });
}

rm_status rm_index_build(rm_ctx* ctx) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!c.have_cloud) return fail(c, RM_ERR_STATE, "rm_index_build: no cloud");
    c.drop_graph();
    if (c.n == 0) {
      c.have_index = true;
      c.depth = 0;
      return RM_OK;
    }
    if (!build_index(c)) return RM_ERR_INVALID;
    CK(cudaStreamSynchronize(c.stream));
    return RM_OK;
  });
}

rm_status rm_knn(rm_ctx* ctx, const float* queries, int32_t stride, int64_t m, int32_t k,
                 int32_t* idx_out, float* d2_out, int32_t loc) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!c.have_index) return fail(c, RM_ERR_STATE, "rm_knn: index not built");
    if (m < 0 || k < 1 || stride < 3 || (m > 0 && (!queries || !idx_out || !d2_out)))
      return fail(c, RM_ERR_INVALID, "rm_knn: bad arguments");
    if (k > 32) return fail(c, RM_ERR_LIMIT, "rm_knn: k above 32");
    if (m == 0) return RM_OK;
    size_t outb = (size_t)m * k;
    const float* dq = (const float*)stage_in(c, c.staging_in, queries, (size_t)m * stride * sizeof(float), loc);
    int32_t* di = idx_out;
    float* dd = d2_out;
    if (loc == RM_HOST) {
      c.staging_out.reserve(outb * 8);
      di = c.staging_out.ptr<int32_t>();
      dd = reinterpret_cast<float*>(c.staging_out.ptr<int32_t>() + outb);
    }
    if (c.n == 0) {
      // empty cloud: all rows padded
      std::vector<int32_t> hi(outb, -1);
      std::vector<float> hd(outb, INFINITY);
      CK(cudaMemcpyAsync(di, hi.data(), outb * 4, cudaMemcpyHostToDevice, c.stream));
      CK(cudaMemcpyAsync(dd, hd.data(), outb * 4, cudaMemcpyHostToDevice, c.stream));
      CK(cudaStreamSynchronize(c.stream));
    } else {
      CK(cudaMemsetAsync(err_counter(c), 0, 8, c.stream));
      launch_knn(c, dq, stride, m, k, di, dd);
      CK(cudaGetLastError());
    }
    if (loc == RM_HOST) {
      CK(cudaMemcpyAsync(idx_out, di, outb * 4, cudaMemcpyDeviceToHost, c.stream));
      CK(cudaMemcpyAsync(d2_out, dd, outb * 4, cudaMemcpyDeviceToHost, c.stream));
      if (c.n > 0) check_kernel_errors(c);
      CK(cudaStreamSynchronize(c.stream));
    }
    return RM_OK;
  });
}

rm_status rm_radii_compute(rm_ctx* ctx, float max_radius, float* radii_out, int32_t* nn_out,
                           int32_t loc) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!c.have_index) return fail(c, RM_ERR_STATE, "rm_radii_compute: index not built");
    if (!std::isfinite(max_radius)) return fail(c, RM_ERR_INVALID, "rm_radii_compute: max_radius not finite");
    c.drop_graph();
    size_t n = (size_t)c.n;
    c.radii_clamped.reserve((n ? n : 1) * 4);
    if (n == 0) {
      c.have_radii = true;
      return RM_OK;
    }
    float* dr = radii_out;
    int32_t* dn = nn_out;
    if (loc == RM_HOST) {
      c.staging_out.reserve(n * 8);
      dr = radii_out ? c.staging_out.ptr<float>() : nullptr;
      dn = nn_out ? reinterpret_cast<int32_t*>(c.staging_out.ptr<float>() + n) : nullptr;
    }
    CK(cudaMemsetAsync(err_counter(c), 0, 8, c.stream));
    launch_radii(c, max_radius, dr, dn);  // also sets the records' radii
    CK(cudaGetLastError());
    refresh_max_radius(c);
    check_kernel_errors(c);
    if (loc == RM_HOST) {
      if (radii_out) CK(cudaMemcpyAsync(radii_out, dr, n * 4, cudaMemcpyDeviceToHost, c.stream));
      if (nn_out) CK(cudaMemcpyAsync(nn_out, dn, n * 4, cudaMemcpyDeviceToHost, c.stream));
      CK(cudaStreamSynchronize(c.stream));
    }
    c.have_radii = true;
    return RM_OK;
  });
}

rm_status rm_radii_set(rm_ctx* ctx, const float* radii, int64_t n, float max_radius, int32_t loc) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!c.have_cloud) return fail(c, RM_ERR_STATE, "rm_radii_set: no cloud");
    if (n != c.n)  // main.cu:137-141
      return fail(c, RM_ERR_INVALID, "rm_radii_set: the radii do not contain the same number of points as the cloud");
    if (n > 0 && !radii) return fail(c, RM_ERR_INVALID, "rm_radii_set: null radii");
    c.drop_graph();
    c.radii_clamped.reserve((size_t)(n ? n : 1) * 4);
    if (n > 0) {
      const float* d = (const float*)stage_in(c, c.staging_in, radii, (size_t)n * 4, loc);
      if (c.have_index) {
        launch_clamp_radii(c, d, max_radius);
      } else {
        // clamp only; the index build gathers the radii into the records
        launch_clamp_radii_only(c, d, max_radius);
      }
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(c.stream));
    }
    c.have_radii = true;
    return RM_OK;
  });
}

rm_status rm_view_pane(rm_ctx* ctx, const rm_view* views, int32_t n, float* pane_out) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (n < 0 || (n > 0 && (!views || !pane_out))) return fail(c, RM_ERR_INVALID, "rm_view_pane: bad arguments");
    if (n == 0) return RM_OK;
    c.staging_in.reserve((size_t)n * sizeof(rm_view));
    c.staging_out.reserve((size_t)n * 4);
    CK(cudaMemcpyAsync(c.staging_in.p, views, (size_t)n * sizeof(rm_view), cudaMemcpyHostToDevice, c.stream));
    launch_view_pane(c, c.staging_in.ptr<rm_view>(), n, c.staging_out.ptr<float>());
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(pane_out, c.staging_out.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return RM_OK;
  });
}

rm_status rm_render(rm_ctx* ctx, const rm_view* view, const rm_frame* out, int32_t loc) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!view || !out) return fail(c, RM_ERR_INVALID, "rm_render: null view or frame");
    if (!c.have_index || !c.have_radii)
      return fail(c, RM_ERR_STATE, "rm_render: index and radii must be ready");
    std::string why;
    if (!view_ok(*view, &why)) return fail(c, RM_ERR_INVALID, "rm_render: " + why);
    size_t npix = (size_t)view->width * view->height;
    FrameStaging f{(float4*)out->rgbd, out->hit, out->depth, out->steps};
    const bool direct = loc == RM_HOST && c.n > 0 && frame_pinned(*out, &f);
    if (loc == RM_HOST && !direct) {
      c.frame_bufs.reserve(npix * 28);
      char* b = c.frame_bufs.ptr<char>();
      f.rgbd = out->rgbd ? (float4*)b : nullptr;
      f.hit = out->hit ? (int32_t*)(b + npix * 16) : nullptr;
      f.depth = out->depth ? (float*)(b + npix * 20) : nullptr;
      f.steps = out->steps ? (int32_t*)(b + npix * 24) : nullptr;
    }
    CK(cudaMemsetAsync(counters(c), 0, kCounters * 8, c.stream));
    CK(cudaMemsetAsync(err_counter(c), 0, 8, c.stream));
    c.stats_from_noalloc = false;
    if (c.n == 0) {
      // empty cloud: every ray misses (no candidate ever comes within MIN_DIST)
      if (f.rgbd) CK(cudaMemsetAsync(f.rgbd, 0, npix * 16, c.stream));
      if (f.hit) CK(cudaMemsetAsync(f.hit, 0xff, npix * 4, c.stream));
      if (f.depth) CK(cudaMemsetAsync(f.depth, 0, npix * 4, c.stream));
      if (f.steps) CK(cudaMemsetAsync(f.steps, 0, npix * 4, c.stream));
    } else {
      CK(cudaEventRecord(c.ev0, c.stream));
      launch_render_plain(c, *view, f.rgbd, f.hit, f.depth, f.steps, counters(c));
      CK(cudaGetLastError());
      CK(cudaEventRecord(c.ev1, c.stream));
    }
    if (loc == RM_HOST) {
      if (!direct) {
        if (out->rgbd) CK(cudaMemcpyAsync(out->rgbd, f.rgbd, npix * 16, cudaMemcpyDeviceToHost, c.stream));
        if (out->hit) CK(cudaMemcpyAsync(out->hit, f.hit, npix * 4, cudaMemcpyDeviceToHost, c.stream));
        if (out->depth) CK(cudaMemcpyAsync(out->depth, f.depth, npix * 4, cudaMemcpyDeviceToHost, c.stream));
        if (out->steps) CK(cudaMemcpyAsync(out->steps, f.steps, npix * 4, cudaMemcpyDeviceToHost, c.stream));
      }
      check_kernel_errors(c);
    }
    c.stats.kernel_ms = -1.0f;
    return RM_OK;
  });
}

}  // extern "C"

namespace {

// Host-side ViewDev table for a batch; returns the number of work items.
int64_t fill_views(Ctx& c, const rm_view* views, int n, const rm_launch& L, ViewDev* hv,
                   int64_t* pix_base) {
  int64_t items = 0, pix = 0;
  for (int v = 0; v < n; ++v) {
    ViewDev& d = hv[v];
    memset(&d, 0, sizeof(d));
    memcpy(d.m, views[v].cam2world, sizeof(d.m));
    d.width = views[v].width;
    d.height = views[v].height;
    d.fov = views[v].fov;
    d.pane = 0.0f;
    d.tiles_x = (d.width + L.tile_w - 1) / L.tile_w;
    int ih = L.tile_h * L.rays_per_lane;
    d.tiles_y = (d.height + ih - 1) / ih;
    d.tile_base = items;
    items += (int64_t)d.tiles_x * d.tiles_y;
    if (pix_base) pix_base[v] = pix;
    pix += (int64_t)d.width * d.height;
  }
  if (pix_base) pix_base[n] = pix;
  return items;
}

void ensure_pinned(Ctx& c, size_t bytes) {
  if (bytes <= c.pinned_views_cap) return;
  if (c.pinned_views) {
    // a captured graph may still read the old buffer
    CK(cudaStreamSynchronize(c.stream));
    c.drop_graph();
    CK(cudaFreeHost(c.pinned_views));
  }
  c.pinned_views = nullptr;
  c.pinned_views_cap = 0;
  CK(cudaMallocHost(&c.pinned_views, bytes));
  c.pinned_views_cap = bytes;
}

// Enqueue one batched render of the views already in c.pinned_views.
void enqueue_batch(Ctx& c, int n, int64_t items, const rm_launch& L) {
  size_t vbytes = (size_t)n * sizeof(ViewDev);
  bool key_ok = c.graph_exec && c.graph_key_n == n && c.graph_key_views == (void*)(intptr_t)items &&
                c.graph_key_launch.tile_w == L.tile_w && c.graph_key_launch.tile_h == L.tile_h &&
                c.graph_key_launch.rays_per_lane == L.rays_per_lane &&
                c.graph_key_launch.ctas_per_sm == L.ctas_per_sm &&
                c.graph_key_launch.search == L.search;
  if (!key_ok) {
    c.drop_graph();
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    CK(cudaMemcpyAsync(c.views.p, c.pinned_views, vbytes, cudaMemcpyHostToDevice, c.stream));
    launch_prepare_views(c, c.views.ptr<ViewDev>(), n, counters(c));
    CK(cudaMemsetAsync(c.queue.p, 0, 8, c.stream));
    CK(cudaMemsetAsync(counters(c), 0, kCounters * 8, c.stream));
    CK(cudaMemsetAsync(err_counter(c), 0, 8, c.stream));
    launch_render_batch(c, c.views.ptr<ViewDev>(), n, items, L, c.queue.ptr<unsigned long long>(), counters(c));
    cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    if (e != cudaSuccess) throw CudaError(std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&c.graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      c.graph_exec = nullptr;
      throw CudaError(std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    c.graph_key_n = n;
    c.graph_key_views = (void*)(intptr_t)items;
    c.graph_key_launch = L;
  }
  // timing events go on the stream around the graph (event nodes inside a
  // graph cannot be used for elapsed-time queries)
  CK(cudaEventRecord(c.ev0, c.stream));
  CK(cudaGraphLaunch(c.graph_exec, c.stream));
  CK(cudaEventRecord(c.ev1, c.stream));
}

bool launch_ok(const rm_launch& L) {
  return L.tile_w > 0 && L.tile_h > 0 && L.tile_w * L.tile_h == 32 && L.rays_per_lane >= 1 &&
         L.rays_per_lane <= 16 && L.ctas_per_sm >= 1 && L.ctas_per_sm <= 16 &&
         (L.search == 0 || L.search == 1);
}

}  // namespace

extern "C" {

rm_status rm_render_batch(rm_ctx* ctx, const rm_view* views, int32_t n, const rm_frame* out,
                          int32_t loc) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (n < 0 || (n > 0 && (!views || !out))) return fail(c, RM_ERR_INVALID, "rm_render_batch: bad arguments");
    if (!c.have_index || !c.have_radii)
      return fail(c, RM_ERR_STATE, "rm_render_batch: index and radii must be ready");
    if (n == 0) return RM_OK;
    std::string why;
    for (int v = 0; v < n; ++v)
      if (!view_ok(views[v], &why)) return fail(c, RM_ERR_INVALID, "rm_render_batch: view " + std::to_string(v) + ": " + why);
    if (c.n == 0) {
      for (int v = 0; v < n; ++v) {
        rm_status s = rm_render(ctx, &views[v], &out[v], loc);
        if (s != RM_OK) return s;
      }
      return RM_OK;
    }
    // previous replay may still read the pinned view table
    CK(cudaEventSynchronize(c.ev1));
    ensure_pinned(c, (size_t)n * sizeof(ViewDev));
    ViewDev* hv = (ViewDev*)c.pinned_views;
    std::vector<int64_t> base(n + 1);
    int64_t items = fill_views(c, views, n, c.launch, hv, base.data());
    int64_t total = base[n];
    bool direct = loc == RM_HOST;
    for (int v = 0; direct && v < n; ++v) {
      FrameStaging f;
      if (!frame_pinned(out[v], &f)) {
        direct = false;
        break;
      }
      hv[v].rgbd = f.rgbd;
      hv[v].hit = f.hit;
      hv[v].depth = f.depth;
      hv[v].steps = f.steps;
    }
    if (loc == RM_HOST && !direct) {
      c.frame_bufs.reserve((size_t)total * 28);
      char* b = c.frame_bufs.ptr<char>();
      for (int v = 0; v < n; ++v) {
        size_t o = (size_t)base[v];
        hv[v].rgbd = out[v].rgbd ? (float4*)(b + o * 16) : nullptr;
        hv[v].hit = out[v].hit ? (int32_t*)(b + (size_t)total * 16 + o * 4) : nullptr;
        hv[v].depth = out[v].depth ? (float*)(b + (size_t)total * 20 + o * 4) : nullptr;
        hv[v].steps = out[v].steps ? (int32_t*)(b + (size_t)total * 24 + o * 4) : nullptr;
      }
    } else if (loc != RM_HOST) {
      for (int v = 0; v < n; ++v) {
        hv[v].rgbd = (float4*)out[v].rgbd;
        hv[v].hit = out[v].hit;
        hv[v].depth = out[v].depth;
        hv[v].steps = out[v].steps;
      }
    }
    c.views.reserve((size_t)n * sizeof(ViewDev));
    enqueue_batch(c, n, items, c.launch);
    c.stats_from_noalloc = false;
    if (loc == RM_HOST) {
      for (int v = 0; !direct && v < n; ++v) {
        size_t np = (size_t)views[v].width * views[v].height;
        if (out[v].rgbd) CK(cudaMemcpyAsync(out[v].rgbd, hv[v].rgbd, np * 16, cudaMemcpyDeviceToHost, c.stream));
        if (out[v].hit) CK(cudaMemcpyAsync(out[v].hit, hv[v].hit, np * 4, cudaMemcpyDeviceToHost, c.stream));
        if (out[v].depth) CK(cudaMemcpyAsync(out[v].depth, hv[v].depth, np * 4, cudaMemcpyDeviceToHost, c.stream));
        if (out[v].steps) CK(cudaMemcpyAsync(out[v].steps, hv[v].steps, np * 4, cudaMemcpyDeviceToHost, c.stream));
      }
      check_kernel_errors(c);
    }
    c.stats.kernel_ms = -1.0f;
    return RM_OK;
  });
}

rm_status rm_set_launch(rm_ctx* ctx, const rm_launch* launch) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!launch || !launch_ok(*launch)) return fail(c, RM_ERR_INVALID, "rm_set_launch: tile_w*tile_h must be 32, 1<=rays_per_lane<=16, 1<=ctas_per_sm<=16, search 0 or 1");
    c.launch = *launch;
    c.drop_graph();
    return RM_OK;
  });
}

rm_status rm_get_launch(rm_ctx* ctx, rm_launch* launch) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!launch) return fail(c, RM_ERR_INVALID, "rm_get_launch: null");
    *launch = c.launch;
    return RM_OK;
  });
}

rm_status rm_get_stats(rm_ctx* ctx, rm_stats* stats) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (!stats) return fail(c, RM_ERR_INVALID, "rm_get_stats: null");
    if (c.stats_from_noalloc) {
      *stats = rm_stats{};
      return RM_OK;
    }
    unsigned long long h[kCounters];
    CK(cudaMemcpyAsync(h, counters(c), sizeof(h), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, c.ev0, c.ev1) != cudaSuccess) {
      cudaGetLastError();
      ms = 0.0f;
    }
    c.stats.steps = (int64_t)h[0];
    c.stats.rays = (int64_t)h[1];
    c.stats.hits = (int64_t)h[2];
    c.stats.packet_steps = (int64_t)h[4];
    c.stats.solo_steps = (int64_t)h[5];
    c.stats.packet_leaves = (int64_t)h[6];
    c.stats.packet_nodes = (int64_t)h[7];
    c.stats.warp_steps = (int64_t)h[8];
    c.stats.split_steps = (int64_t)h[9];
    c.stats.search_errors = (int64_t)h[3];
    c.stats.queue_spills = (int64_t)h[10];
    c.stats.dfs_walks = (int64_t)h[11];
    c.stats.kernel_ms = ms;
    *stats = c.stats;
    return RM_OK;
  });
}

rm_status rm_backward(rm_ctx* ctx, const rm_view* views, int32_t n, const float* dl_drgb,
                      const float* dl_ddepth, const int32_t* hit, float* g_rgb, float* g_xyz,
                      float* g_radius, int32_t loc) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (n < 0 || (n > 0 && (!views || !dl_drgb || !dl_ddepth || !hit || !g_rgb || !g_xyz || !g_radius)))
      return fail(c, RM_ERR_INVALID, "rm_backward: bad arguments");
    if (!c.have_index || !c.have_radii) return fail(c, RM_ERR_STATE, "rm_backward: index and radii must be ready");
    if (n == 0 || c.n == 0) return RM_OK;
    std::string why;
    for (int v = 0; v < n; ++v)
      if (!view_ok(views[v], &why)) return fail(c, RM_ERR_INVALID, "rm_backward: view " + std::to_string(v) + ": " + why);
    std::vector<ViewDev> hv(n);
    std::vector<int64_t> base(n + 1);
    fill_views(c, views, n, c.launch, hv.data(), base.data());
    int64_t total = base[n];
    size_t vb = (size_t)n * sizeof(ViewDev), bb = (size_t)(n + 1) * 8;
    // table layout in staging_in: views | pix_base | (host inputs)
    size_t off_in = ((vb + bb + 255) / 256) * 256;
    size_t need_in = off_in + (loc == RM_HOST ? (size_t)total * 20 : 0);
    c.staging_in.reserve(need_in);
    char* si = c.staging_in.ptr<char>();
    ViewDev* dv = (ViewDev*)si;
    int64_t* db = (int64_t*)(si + vb);
    CK(cudaMemcpyAsync(dv, hv.data(), vb, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(db, base.data(), bb, cudaMemcpyHostToDevice, c.stream));
    launch_prepare_views(c, dv, n, counters(c));
    const float* drgb = dl_drgb;
    const float* ddep = dl_ddepth;
    const int32_t* dhit = hit;
    float *gr = g_rgb, *gx = g_xyz, *gd = g_radius;
    size_t np = (size_t)c.n;
    if (loc == RM_HOST) {
      float* p = (float*)(si + off_in);
      CK(cudaMemcpyAsync(p, dl_drgb, (size_t)total * 12, cudaMemcpyHostToDevice, c.stream));
      CK(cudaMemcpyAsync(p + 3 * total, dl_ddepth, (size_t)total * 4, cudaMemcpyHostToDevice, c.stream));
      CK(cudaMemcpyAsync(p + 4 * total, hit, (size_t)total * 4, cudaMemcpyHostToDevice, c.stream));
      drgb = p;
      ddep = p + 3 * total;
      dhit = (const int32_t*)(p + 4 * total);
      c.staging_out.reserve(np * 28);
      gr = c.staging_out.ptr<float>();
      gx = gr + 3 * np;
      gd = gx + 3 * np;
      CK(cudaMemcpyAsync(gr, g_rgb, np * 12, cudaMemcpyHostToDevice, c.stream));
      CK(cudaMemcpyAsync(gx, g_xyz, np * 12, cudaMemcpyHostToDevice, c.stream));
      CK(cudaMemcpyAsync(gd, g_radius, np * 4, cudaMemcpyHostToDevice, c.stream));
    }
    launch_backward(c, dv, n, total, db, drgb, ddep, dhit, gr, gx, gd);
    CK(cudaGetLastError());
    if (loc == RM_HOST) {
      CK(cudaMemcpyAsync(g_rgb, gr, np * 12, cudaMemcpyDeviceToHost, c.stream));
      CK(cudaMemcpyAsync(g_xyz, gx, np * 12, cudaMemcpyDeviceToHost, c.stream));
      CK(cudaMemcpyAsync(g_radius, gd, np * 4, cudaMemcpyDeviceToHost, c.stream));
    }
    // staging_in holds the view table that the kernel reads: keep it alive
    CK(cudaStreamSynchronize(c.stream));
    return RM_OK;
  });
}

rm_status rm_autotune(rm_ctx* ctx, const rm_view* views, int32_t n, rm_launch* chosen,
                      int32_t* leaf_size, float* best_ms) {
  return guarded(ctx, [&](Ctx& c) -> rm_status {
    if (n <= 0 || !views) return fail(c, RM_ERR_INVALID, "rm_autotune: need views");
    if (!c.have_index || !c.have_radii || c.n == 0)
      return fail(c, RM_ERR_STATE, "rm_autotune: index and radii must be ready");
    // device scratch frames (hit + rgbd), released at the end
    int64_t total = 0;
    for (int v = 0; v < n; ++v) total += (int64_t)views[v].width * views[v].height;
    DevBuf scratch;
    scratch.reserve((size_t)total * 20);
    std::vector<rm_frame> fr(n);
    int64_t o = 0;
    for (int v = 0; v < n; ++v) {
      fr[v].rgbd = (float*)(scratch.ptr<char>() + o * 16);
      fr[v].hit = (int32_t*)(scratch.ptr<char>() + total * 16 + o * 4);
      fr[v].depth = nullptr;
      fr[v].steps = nullptr;
      o += (int64_t)views[v].width * views[v].height;
    }
    auto time_once = [&](const rm_launch& L) -> float {
      c.launch = L;
      float best = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        rm_status s = rm_render_batch(ctx, views, n, fr.data(), RM_DEVICE);
        if (s != RM_OK) throw std::runtime_error("autotune render failed: " + c.err);
        CK(cudaStreamSynchronize(c.stream));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        best = std::min(best, ms);
      }
      return best;
    };
    // Packet search keeps a tile's rays in lockstep (refilling lanes mid-tile
    // breaks the coherence it lives on), so rays_per_lane > 1 is tried with
    // the per-ray walk only.
    const int shapes[3][2] = {{8, 4}, {4, 8}, {16, 2}};
    rm_launch best_l = c.launch;
    float best_t = 1e30f;
    // A candidate replaces the incumbent only when it is at least 1% faster:
    // the launch shapes near the optimum differ by about that much, less than
    // the tail of a short timing batch moves them (the last items of the
    // queue leave SMs idle), and the first candidate of each group is the
    // one measured best on full-size batches.
    auto better = [&](float t) { return t < best_t * 0.99f; };
    for (auto& sh : shapes) {
      rm_launch L{sh[0], sh[1], 1, 8, 1};
      float t = time_once(L);
      if (best_t >= 1e30f || better(t)) { best_t = t; best_l = L; }
    }
    for (int ctas : {7, 6, 5}) {
      rm_launch L = best_l;
      L.ctas_per_sm = ctas;
      float t = time_once(L);
      if (better(t)) { best_t = t; best_l = L; }
    }
    for (int rpl : {1, 2}) {
      rm_launch L{best_l.tile_w, best_l.tile_h, rpl, 4, 0};
      float t = time_once(L);
      if (better(t)) { best_t = t; best_l = L; }
    }
    const int start_leaf = c.cfg.leaf_size;
    int best_leaf = start_leaf;
    for (int leaf : {8, 16, 32}) {
      if (leaf == start_leaf) continue;
      c.cfg.leaf_size = leaf;
      c.drop_graph();
      if (!build_index(c)) throw std::runtime_error(c.err);
      float t = time_once(best_l);
      if (better(t)) {
        best_t = t;
        best_leaf = leaf;
      }
    }
    if (c.cfg.leaf_size != best_leaf) {
      c.cfg.leaf_size = best_leaf;
      c.drop_graph();
      if (!build_index(c)) throw std::runtime_error(c.err);
    }
    CK(cudaStreamSynchronize(c.stream));
    scratch.release();
    c.launch = best_l;
    c.drop_graph();
    if (chosen) *chosen = best_l;
    if (leaf_size) *leaf_size = best_leaf;
    if (best_ms) *best_ms = best_t;
    return RM_OK;
  });
}

}  // extern "C"
