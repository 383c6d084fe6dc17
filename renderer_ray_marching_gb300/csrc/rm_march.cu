// rm_march.cu -- the sphere-tracing marcher (replaces the reference's
// render kernel, src/ray_marching.cu:63-91, and its per-step FLANN query,
// :202-292).
//
// Plain form (rm_render): one thread per pixel, 128-thread CTAs made of four
// warps, each warp an 8x4 pixel tile so its 32 rays are screen neighbours
// and walk the same part of the tree.  No per-pixel scratch in global
// memory: the 10-NN list lives in registers (the reference keeps a 10-entry
// index/distance array and the query point per pixel in global memory,
// src/ray_marching.cu:98-103, 266-278).
//
// Batched form (rm_render_batch): a persistent kernel, ctas_per_sm CTAs per
// SM, whose warps pull work items (tile_w x tile_h*rays_per_lane pixels of
// one view) from a global counter.  Each lane marches one ray at a time;
// after every distance step the warp votes (__ballot_sync) which lanes have
// retired their ray and refills exactly those lanes from the warp's current
// item, taking a new item when it runs dry.  Lanes therefore stay busy
// regardless of how unevenly step counts are spread over a tile or over
// views of different sizes.
//
// Culling.  The reference's view-frustum test is a no-op (is_inside,
// src/ray_marching.cu:231-258, returns true); its effective culling is the
// near-plane start and the far-plane stop.  Here each ray additionally gets
// an exact exit bound: let E be the box of all sphere centres grown by
// (max radius + MIN_DIST + slack).  Every step position beyond the ray's
// exit from E is farther than max radius + MIN_DIST from every centre, so
// every later distance value exceeds MIN_DIST (and is positive, so t keeps
// growing): the reference would march on to the far plane or the step cap
// and report a miss.  Stopping at the exit therefore never changes an
// output, it only skips work.  The slack (2e-3 m plus 1e-6 of the scene
// scale) covers float rounding of positions and distances.
#include "rm_internal.h"

namespace rm {

struct ClipBox {
  float lo[3], hi[3];
};

// Exit parameter of the ray from box E (-inf if the ray never meets E).
__device__ __forceinline__ float clip_exit(const Ray& r, const ClipBox& e) {
  float o[3] = {r.ox, r.oy, r.oz}, d[3] = {r.dx, r.dy, r.dz};
  float tmin = -INFINITY, tmax = INFINITY;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (d[a] != 0.0f) {
      float inv = 1.0f / d[a];
      float t1 = (e.lo[a] - o[a]) * inv, t2 = (e.hi[a] - o[a]) * inv;
      tmin = fmaxf(tmin, fminf(t1, t2));
      tmax = fminf(tmax, fmaxf(t1, t2));
    } else if (o[a] < e.lo[a] || o[a] > e.hi[a]) {
      tmax = -INFINITY;
    }
  }
  if (!(tmin <= tmax)) return -INFINITY;
  // outward slack for the rounding of the slab divisions
  return tmax + fabsf(tmax) * 1e-5f + 1e-3f;
}

struct PlainArgs {
  float m[16];
  int32_t width, height;
  float fov;
  ClipBox clip;
  float4* rgbd;
  int32_t* hit;
  float* depth;
  int32_t* steps;
};

__device__ __forceinline__ void write_result(const IndexDev& ix, const MarchResult& mr, int64_t pix,
                                             float4* rgbd, int32_t* hit, float* depth,
                                             int32_t* steps) {
  if (mr.s >= 0) {
    float4 c = __ldg(ix.col + mr.s);
    c.w = mr.depth;  // colour with the depth in .w (src/ray_marching.cu:85-89)
    if (rgbd) rgbd[pix] = c;
    if (hit) hit[pix] = __ldg(ix.perm + mr.s);
    if (depth) depth[pix] = mr.depth;
  } else {
    if (rgbd) rgbd[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // BACKGROUND_COLOR
    if (hit) hit[pix] = -1;
    if (depth) depth[pix] = 0.0f;
  }
  if (steps) steps[pix] = mr.steps;
}

// counters: [0] steps, [1] rays, [2] culled rays, [3] search errors
__global__ void __launch_bounds__(128)
k_march_plain(IndexDev ix, PlainArgs a, unsigned long long* __restrict__ counters) {
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  int y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
  bool active = x < a.width && y < a.height;
  unsigned steps = 0, bad = 0;
  if (active) {
    float pane = view_pane(a.width, a.fov);
    Ray r = make_ray(a.m, a.width, a.height, pane, x, y);
    float t_stop = clip_exit(r, a.clip);
    MarchResult mr = march_ray(ix, r, t_stop);
    write_result(ix, mr, (int64_t)y * a.width + x, a.rgbd, a.hit, a.depth, a.steps);
    steps = (unsigned)mr.steps;
    bad = mr.ok ? 0u : 1u;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    steps += __shfl_xor_sync(0xffffffffu, steps, off);
    bad += __shfl_xor_sync(0xffffffffu, bad, off);
  }
  unsigned nact = __popc(__ballot_sync(0xffffffffu, active));
  if (lane == 0) {
    atomicAdd(counters + 0, (unsigned long long)steps);
    atomicAdd(counters + 1, (unsigned long long)nact);
    if (bad) atomicAdd(counters + 3, (unsigned long long)bad);
  }
}

// ---------------------------------------------------------------- batched
__global__ void k_prepare_views(ViewDev* __restrict__ views, int n) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) views[v].pane = view_pane(views[v].width, views[v].fov);
}

__global__ void k_view_pane(const rm_view* __restrict__ views, int n, float* __restrict__ out) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) out[v] = view_pane(views[v].width, views[v].fov);
}

struct BatchArgs {
  const ViewDev* views;
  int nviews;
  int64_t total_items;
  int tile_w, tile_h, rpl;  // item = tile_w x (tile_h * rpl) pixels
  ClipBox clip;
};

__device__ __forceinline__ int find_view(const ViewDev* views, int n, int64_t item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (views[mid].tile_base <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(128)
k_march_batch(IndexDev ix, BatchArgs a, unsigned long long* __restrict__ queue,
              unsigned long long* __restrict__ counters) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int item_rays = a.tile_w * a.tile_h * a.rpl;
  // warp-uniform pool state
  int next = item_rays;
  int iv = 0, ix0 = 0, iy0 = 0;
  bool pool_open = true;
  // lane ray state
  bool has = false;
  int view = 0;
  int64_t pix = 0;
  Ray r;
  float t = 0.0f, t_stop = 0.0f;
  int nsteps = 0;
  KList<KNN> L;  // the lane's neighbours from its previous step
  unsigned long long steps_total = 0, rays_total = 0, bad = 0;

  while (true) {
    unsigned need = __ballot_sync(FULL, !has);
    while (need && pool_open) {
      if (next >= item_rays) {
        unsigned long long it = 0;
        if (lane == 0) it = atomicAdd(queue, 1ull);
        it = __shfl_sync(FULL, it, 0);
        if ((int64_t)it >= a.total_items) {
          pool_open = false;
          break;
        }
        iv = find_view(a.views, a.nviews, (int64_t)it);
        const ViewDev& V = a.views[iv];
        int64_t local = (int64_t)it - V.tile_base;
        ix0 = (int)(local % V.tiles_x) * a.tile_w;
        iy0 = (int)(local / V.tiles_x) * (a.tile_h * a.rpl);
        next = 0;
      }
      int idx = next + __popc(need & lt);
      if (!has && idx < item_rays) {
        const ViewDev& V = a.views[iv];
        int x = ix0 + idx % a.tile_w;
        int y = iy0 + idx / a.tile_w;
        if (x < V.width && y < V.height) {
          has = true;
          view = iv;
          pix = (int64_t)y * V.width + x;
          r = make_ray(V.m, V.width, V.height, V.pane, x, y);
          t_stop = clip_exit(r, a.clip);
          t = r.t_near;
          nsteps = 0;
          klist_init<KNN>(L);
        }
      }
      next += __popc(need);
      need = __ballot_sync(FULL, !has);
    }
    if (__ballot_sync(FULL, has) == 0) break;
    if (has) {
      // one step of src/ray_marching.cu:215-225
      bool done = false;
      MarchResult mr;
      mr.s = -1;
      mr.depth = 0.0f;
      if (t > t_stop) {
        done = true;  // culled: cannot hit any more
      } else {
        float px = __fmaf_rn(r.dx, t, r.ox);
        float py = __fmaf_rn(r.dy, t, r.oy);
        float pz = __fmaf_rn(r.dz, t, r.oz);
        int32_t s;
        bool ok;
        float step = distance_step(ix, px, py, pz, L, &s, &ok);
        if (!ok) ++bad;
        ++nsteps;
        t = __fadd_rn(t, step);
        if (step < MIN_DIST) {
          mr.s = s;
          mr.depth = t;
          done = true;
        } else if (t > r.t_far || nsteps >= MAX_STEPS) {
          done = true;
        }
      }
      if (done) {
        const ViewDev& V = a.views[view];
        mr.steps = nsteps;
        mr.ok = true;
        write_result(ix, mr, pix, V.rgbd, V.hit, V.depth, V.steps);
        steps_total += (unsigned long long)nsteps;
        rays_total += 1;
        has = false;
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    steps_total += __shfl_xor_sync(FULL, steps_total, off);
    rays_total += __shfl_xor_sync(FULL, rays_total, off);
    bad += __shfl_xor_sync(FULL, bad, off);
  }
  if (lane == 0) {
    atomicAdd(counters + 0, steps_total);
    atomicAdd(counters + 1, rays_total);
    if (bad) atomicAdd(counters + 3, bad);
  }
}

// ---------------------------------------------------------------- host side
// Box E of the culling argument above; max_r = +inf disables culling.
static ClipBox clip_box(const Ctx& c, float max_r) {
  ClipBox e;
  if (!(max_r < INFINITY)) {
    for (int a = 0; a < 3; ++a) {
      e.lo[a] = -INFINITY;
      e.hi[a] = INFINITY;
    }
    return e;
  }
  float scale = 0.0f;
  for (int a = 0; a < 6; ++a) scale = fmaxf(scale, fabsf(c.bounds[a]));
  float m = max_r + MIN_DIST + 2e-3f + 1e-6f * (scale + ZFAR * 16.0f);
  for (int a = 0; a < 3; ++a) {
    e.lo[a] = c.bounds[a] - m;
    e.hi[a] = c.bounds[3 + a] + m;
  }
  return e;
}

void launch_view_pane(Ctx& c, const rm_view* views_dev, int n, float* pane_out) {
  k_view_pane<<<(n + 127) / 128, 128, 0, c.stream>>>(views_dev, n, pane_out);
}

void launch_render_plain(Ctx& c, const rm_view& v, float4* rgbd, int32_t* hit, float* depth,
                         int32_t* steps, unsigned long long* counters) {
  PlainArgs a;
  memcpy(a.m, v.cam2world, sizeof(a.m));
  a.width = v.width;
  a.height = v.height;
  a.fov = v.fov;
  a.clip = clip_box(c, c.max_r);
  a.rgbd = rgbd;
  a.hit = hit;
  a.depth = depth;
  a.steps = steps;
  dim3 grid((v.width + 15) / 16, (v.height + 7) / 8);
  k_march_plain<<<grid, 128, 0, c.stream>>>(c.index(), a, counters);
}

void launch_prepare_views(Ctx& c, ViewDev* views_dev, int n, unsigned long long* counters) {
  (void)counters;
  k_prepare_views<<<(n + 127) / 128, 128, 0, c.stream>>>(views_dev, n);
}

void launch_render_batch(Ctx& c, ViewDev* views_dev, int n, int64_t total_items, const rm_launch& L,
                         unsigned long long* counters) {
  BatchArgs a;
  a.views = views_dev;
  a.nviews = n;
  a.total_items = total_items;
  a.tile_w = L.tile_w;
  a.tile_h = L.tile_h;
  a.rpl = L.rays_per_lane;
  a.clip = clip_box(c, c.max_r);
  unsigned long long* queue = c.queue.ptr<unsigned long long>();
  int grid = c.sm_count * (L.ctas_per_sm > 0 ? L.ctas_per_sm : 4);
  k_march_batch<<<grid, 128, 0, c.stream>>>(c.index(), a, queue, counters);
}

}  // namespace rm
