// rm_march.cu -- the sphere-tracing marcher (replaces the reference's
// render kernel, src/ray_marching.cu:63-91, and its per-step FLANN query,
// :202-292).
//
// Work unit: one warp marches the rays of a screen tile (tile_w x tile_h
// pixels, 32 rays; with rays_per_lane > 1 an item is rays_per_lane such
// tiles stacked vertically and a lane whose ray ends takes the item's next
// pixel).  Each distance step is an exact 10-NN of every lane's step
// position, found by a warp packet traversal:
//
//   1. seed: every lane re-measures its previous step's 10 points at the new
//      position; the largest of those distances bounds the new 10th distance
//      (they are valid candidates), so its set restarts with that finite
//      bound (KSet::restart);
//   2. the warp walks the tree once, as a unit (packet_knn): a node is
//      expanded when its box lies within the current 10th distance of ANY
//      active lane (one OR-reduction of 4-bit child votes), children are
//      visited nearest-first for a leading lane, and pending nodes wait in a
//      priority queue keyed by the leading lane's box distance
//      (packet_knn_bf);
//   3. a leaf's records are staged once for the whole warp (broadcast
//      loads) and every lane updates its own sorted set, so all lanes'
//      bounds tighten while the walk goes on.
// Neighbouring rays need nearly the same leaves (at surfaces, and in open
// space where the 10 nearest of every lane cluster around the same foot
// point), so the warp pays for the union of their searches once instead of
// serialising 32 divergent walks.  Search mode 0 keeps one independent walk
// per lane.  Then the step value min(sqrtf(d2) - r) and the reference's
// termination tests (MIN_DIST hit, far plane, MAX_STEPS).
//
// Plain form (rm_render): one warp per 8x4 tile, four warps per CTA.
// Batched form (rm_render_batch): a persistent kernel whose warps pull items
// of any view from one global counter; the whole launch is a CUDA graph.
// Both are templated on the CTAs per SM their register cap is sized for
// (4 to 8, regs_for_ctas); the kernel is latency-bound, so resident warps matter and
// the per-item view and the statistics live in shared memory (WarpSmem).
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

#include <cstring>

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

constexpr int WARPS_PER_CTA = 4;

// Register cap of a marcher instance sized for `ctas` resident CTAs per SM:
// the SM's 65,536 registers shared by ctas x 128 threads, rounded down to the
// allocation granule of 8 (4 -> 128, 5 -> 96, 6 -> 80, 7 -> 72, 8 -> 64).
// The kernels take it as __maxnreg__ rather than as the minimum-blocks
// argument of __launch_bounds__: both give ptxas the same register count,
// but it then spills different values, and on the 20M-point batched
// workload (32 views, leaf 16) the capped form measured 54.7 Mrays/s at 64
// and at 72 registers against 48.2 for __launch_bounds__(128, 8).  The
// marcher is latency-bound, so the extra resident warps are worth the
// spills (72 registers: 200 B of spill stores per thread).
constexpr int regs_for_ctas(int ctas) { return (65536 / (ctas * 32 * WARPS_PER_CTA)) / 8 * 8; }

struct MarchParams {
  ClipBox clip;
  int search;  // 1: warp packet traversal, 0: one walk per lane
};

// View as seen by the marcher (kept per warp in shared memory).
struct ViewArgs {
  float m[16];
  int32_t width, height;
  float pane;
  float4* rgbd;
  int32_t* hit;
  float* depth;
  int32_t* steps;
};

// counters: [0] steps, [1] rays, [2] hits, [3] search errors,
//           [4] packet lane-steps, [5] per-lane lane-steps, [6] leaves scanned by packets,
//           [7] nodes expanded by packets, [8] warp steps, [9] warp steps split in two packets
//           (no longer split: always 0), [10] queue entries moved to the overflow stack,
//           [11] packet walks that fell back to depth-first order
enum { C_STEPS, C_RAYS, C_HITS, C_BAD, C_COOP, C_SOLO, C_LEAVES, C_NODES, C_WSTEPS, C_SPLIT, C_SPILL, C_DFS,
       C_N };

// Per-warp shared state.  The view of the current item, the statistics and
// each lane's ray live here rather than in registers: they are read or bumped
// at a ray's start and end, or once per step (the ray's origin, direction and
// t before the walk, t and the step count after it), and every register the
// walk does not have to hold lets more warps stay resident (the marcher is
// bound by instruction latency, so resident warps are what hides it; parking
// the ray here cut the 64-register instance's spills from 314 to 204 B and
// gained 1%).
struct RayLanes {
  float ox[32], oy[32], oz[32], dx[32], dy[32], dz[32];
  float t[32], t_stop[32], t_far[32];
  int32_t nsteps[32], pix[32];
};
struct WarpSmem {
  PacketQueue ps;
  ViewArgs v;                   // warp-uniform; written by lane 0 per item
  unsigned long long cnt[C_N];  // this warp's statistics
  RayLanes ray;
};

__device__ __forceinline__ void write_result(const IndexDev& ix, const ViewArgs& v, int64_t pix, int32_t s,
                                             float depth, int32_t steps, unsigned long long* cnt) {
  atomicAdd(cnt + C_STEPS, (unsigned long long)steps);
  atomicAdd(cnt + C_RAYS, 1ull);
  if (s >= 0) atomicAdd(cnt + C_HITS, 1ull);
  if (s >= 0) {
    float4 c = __ldg(ix.col + s);
    c.w = depth;  // colour with the depth in .w (src/ray_marching.cu:85-89)
    if (v.rgbd) v.rgbd[pix] = c;
    if (v.hit) v.hit[pix] = __ldg(ix.perm + s);
    if (v.depth) v.depth[pix] = depth;
  } else {
    if (v.rgbd) v.rgbd[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // BACKGROUND_COLOR
    if (v.hit) v.hit[pix] = -1;
    if (v.depth) v.depth[pix] = 0.0f;
  }
  if (v.steps) v.steps[pix] = steps;
}

// Marches every ray of one item (origin x0, y0; tile_w x tile_h*rpl pixels)
// of view v.  All 32 lanes call it.  SEARCH: 1 packet traversal, 0 per lane.
template <int SEARCH>
__device__ void march_item(const IndexDev& ix, int x0, int y0, int tile_w, int tile_h, int rpl,
                           const MarchParams& mp, WarpSmem& sm) {
  const ViewArgs& v = sm.v;
  RayLanes& R = sm.ray;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int item_rays = tile_w * tile_h * rpl;
  int next = 0;
  bool has = false;
  KSet L;
  L.clear();
  while (true) {
    // hand unclaimed pixels of the item to lanes without a ray
    unsigned need = __ballot_sync(FULL, !has);
    while (need && next < item_rays) {
      int idx = next + __popc(need & lt);
      if (!has && idx < item_rays) {
        int x = x0 + idx % tile_w;
        int y = y0 + idx / tile_w;
        if (x < v.width && y < v.height) {
          has = true;
          const Ray r = make_ray(v.m, v.width, v.height, v.pane, x, y);
          R.pix[lane] = y * v.width + x;
          R.ox[lane] = r.ox; R.oy[lane] = r.oy; R.oz[lane] = r.oz;
          R.dx[lane] = r.dx; R.dy[lane] = r.dy; R.dz[lane] = r.dz;
          R.t_stop[lane] = clip_exit(r, mp.clip);
          R.t_far[lane] = r.t_far;
          R.t[lane] = r.t_near;
          R.nsteps[lane] = 0;
          L.clear();
        }
      }
      next += __popc(need);
      need = __ballot_sync(FULL, !has);
    }
    if (__ballot_sync(FULL, has) == 0) break;

    float t = R.t[lane];
    bool stepping = has && !(t > R.t_stop[lane]);  // past the exit bound: a miss (culled)
    if (has && !stepping) {
      write_result(ix, v, R.pix[lane], -1, 0.0f, R.nsteps[lane], sm.cnt);
      has = false;
    }
    float px = __fmaf_rn(R.dx[lane], t, R.ox[lane]);
    float py = __fmaf_rn(R.dy[lane], t, R.oy[lane]);
    float pz = __fmaf_rn(R.dz[lane], t, R.oz[lane]);
    if (stepping) L.restart(ix, px, py, pz);
    if (SEARCH == 1) {
      // One packet: every stepping lane walks with the warp.  (A split into
      // a tight and a loose packet helped the depth-first walk; with the
      // best-first order loose lanes no longer steer the walk and the split
      // measured 2% slower.)
      unsigned lv = 0, nd = 0;
      if (!packet_knn_bf(ix, stepping, px, py, pz, L, sm.ps, lv, nd) && stepping) atomicAdd(sm.cnt + C_BAD, 1ull);
      const unsigned any_step = __ballot_sync(FULL, stepping);  // every lane votes
      if (lane == 0) {
        sm.cnt[C_LEAVES] += lv;
        sm.cnt[C_NODES] += nd;
        sm.cnt[C_WSTEPS] += any_step ? 1 : 0;
      }
    } else if (stepping) {
      if (!knn_search(ix, px, py, pz, L)) atomicAdd(sm.cnt + C_BAD, 1ull);
    }
    if (stepping) {
      int32_t s;
      L.order(ix.perm);
      float step = L.step_value(ix, &s);
      const int nsteps = R.nsteps[lane] + 1;
      R.nsteps[lane] = nsteps;
      t = __fadd_rn(R.t[lane], step);
      R.t[lane] = t;
      bool fin = false;
      int32_t hs = -1;
      float hd = 0.0f;
      if (step < MIN_DIST) {  // src/ray_marching.cu:219-222
        fin = true;
        hs = s;
        hd = t;
      } else if (t > R.t_far[lane] || nsteps >= MAX_STEPS) {
        fin = true;
      }
      if (fin) {
        write_result(ix, v, R.pix[lane], hs, hd, nsteps, sm.cnt);
        has = false;
      }
    }
  }
}

__device__ __forceinline__ void clear_counters(WarpSmem& sm) {
  const int lane = threadIdx.x & 31;
  if (lane < C_N) sm.cnt[lane] = 0ull;
  if (lane == 0) {
    sm.ps.n_spill = 0;
    sm.ps.n_dfs = 0;
  }
  __syncwarp();
}

// Adds the warp's statistics to the launch's counters.  Lane-steps are the
// rays' step counts; they are reported as packet or per-lane lane-steps by
// search mode.
template <int SEARCH>
__device__ __forceinline__ void flush_counters(WarpSmem& sm, unsigned long long* counters) {
  __syncwarp();
  const int lane = threadIdx.x & 31;
  if (lane < C_N) {
    unsigned long long v = lane == C_COOP ? (SEARCH == 1 ? sm.cnt[C_STEPS] : 0ull)
                         : lane == C_SOLO ? (SEARCH == 0 ? sm.cnt[C_STEPS] : 0ull)
                         : lane == C_SPILL ? (unsigned long long)sm.ps.n_spill
                         : lane == C_DFS ? (unsigned long long)sm.ps.n_dfs
                         : sm.cnt[lane];
    if (v) atomicAdd(counters + lane, v);
  }
}


struct PlainArgs {
  float m[16];
  int32_t width, height;
  float fov;
  float4* rgbd;
  int32_t* hit;
  float* depth;
  int32_t* steps;
};

// One warp per 8x4 tile.
template <int SEARCH>
__device__ __forceinline__ void plain_body(const IndexDev& ix, const PlainArgs& a, const MarchParams& mp,
                                           unsigned long long* __restrict__ counters) {
  __shared__ WarpSmem smem[WARPS_PER_CTA];
  const int warp = threadIdx.x >> 5;
  int tiles_x = (a.width + 7) / 8;
  int tile = blockIdx.x * WARPS_PER_CTA + warp;
  int tiles = tiles_x * ((a.height + 3) / 4);
  WarpSmem& sm = smem[warp];
  clear_counters(sm);
  if (tile < tiles) {
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
      for (int k = 0; k < 16; ++k) sm.v.m[k] = a.m[k];
      sm.v.width = a.width;
      sm.v.height = a.height;
      sm.v.pane = view_pane(a.width, a.fov);
      sm.v.rgbd = a.rgbd;
      sm.v.hit = a.hit;
      sm.v.depth = a.depth;
      sm.v.steps = a.steps;
    }
    __syncwarp();
    march_item<SEARCH>(ix, (tile % tiles_x) * 8, (tile / tiles_x) * 4, 8, 4, 1, mp, sm);
  }
  flush_counters<SEARCH>(sm, counters);
}

// Packet-walk instances, MINB: the CTAs per SM their register cap is sized
// for (the launch's ctas_per_sm picks the instance).  The per-lane walk keeps
// the minimum-blocks form, under which it measured faster (20.0 against
// 17.2 Mrays/s with __maxnreg__ at the same 90 registers).
template <int MINB>
__global__ void __launch_bounds__(32 * WARPS_PER_CTA) __maxnreg__(regs_for_ctas(MINB))
k_march_plain(IndexDev ix, PlainArgs a, MarchParams mp, unsigned long long* __restrict__ counters) {
  plain_body<1>(ix, a, mp, counters);
}
__global__ void __launch_bounds__(32 * WARPS_PER_CTA, 4)
k_march_plain_lane(IndexDev ix, PlainArgs a, MarchParams mp, unsigned long long* __restrict__ counters) {
  plain_body<0>(ix, a, mp, counters);
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

template <int SEARCH>
__device__ __forceinline__ void batch_body(const IndexDev& ix, const BatchArgs& a, const MarchParams& mp,
                                           unsigned long long* __restrict__ queue,
                                           unsigned long long* __restrict__ counters) {
  __shared__ WarpSmem smem[WARPS_PER_CTA];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpSmem& sm = smem[warp];
  clear_counters(sm);
  while (true) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(queue, 1ull);
    it = __shfl_sync(0xffffffffu, it, 0);
    if ((int64_t)it >= a.total_items) break;
    int iv = find_view(a.views, a.nviews, (int64_t)it);
    const ViewDev& V = a.views[iv];
    int64_t local = (int64_t)it - V.tile_base;
    __syncwarp();  // the previous item's readers of sm.v are done
    if (lane < 16) sm.v.m[lane] = V.m[lane];
    if (lane == 0) {
      sm.v.width = V.width;
      sm.v.height = V.height;
      sm.v.pane = V.pane;
      sm.v.rgbd = V.rgbd;
      sm.v.hit = V.hit;
      sm.v.depth = V.depth;
      sm.v.steps = V.steps;
    }
    __syncwarp();
    int x0 = (int)(local % V.tiles_x) * a.tile_w;
    int y0 = (int)(local / V.tiles_x) * (a.tile_h * a.rpl);
    march_item<SEARCH>(ix, x0, y0, a.tile_w, a.tile_h, a.rpl, mp, sm);
  }
  flush_counters<SEARCH>(sm, counters);
}

template <int MINB>
__global__ void __launch_bounds__(32 * WARPS_PER_CTA) __maxnreg__(regs_for_ctas(MINB))
k_march_batch(IndexDev ix, BatchArgs a, MarchParams mp, unsigned long long* __restrict__ queue,
              unsigned long long* __restrict__ counters) {
  batch_body<1>(ix, a, mp, queue, counters);
}
__global__ void __launch_bounds__(32 * WARPS_PER_CTA, 4)
k_march_batch_lane(IndexDev ix, BatchArgs a, MarchParams mp, unsigned long long* __restrict__ queue,
                   unsigned long long* __restrict__ counters) {
  batch_body<0>(ix, a, mp, queue, counters);
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

static MarchParams march_params(const Ctx& c) {
  MarchParams mp;
  mp.clip = clip_box(c, c.max_r);
  mp.search = c.launch.search;
  return mp;
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
  a.rgbd = rgbd;
  a.hit = hit;
  a.depth = depth;
  a.steps = steps;
  int64_t tiles = (int64_t)((v.width + 7) / 8) * ((v.height + 3) / 4);
  unsigned grid = (unsigned)((tiles + WARPS_PER_CTA - 1) / WARPS_PER_CTA);
  MarchParams mp = march_params(c);
  auto go = [&](auto kern) { kern<<<grid, 32 * WARPS_PER_CTA, 0, c.stream>>>(c.index(), a, mp, counters); };
  const int cps = c.launch.ctas_per_sm;
  if (mp.search == 1) {
    if (cps >= 8) go(k_march_plain<8>);
    else if (cps >= 7) go(k_march_plain<7>);
    else if (cps >= 6) go(k_march_plain<6>);
    else if (cps >= 5) go(k_march_plain<5>);
    else go(k_march_plain<4>);
  } else {
    go(k_march_plain_lane);
  }
}

void launch_prepare_views(Ctx& c, ViewDev* views_dev, int n, unsigned long long* counters) {
  (void)counters;
  k_prepare_views<<<(n + 127) / 128, 128, 0, c.stream>>>(views_dev, n);
}

// `queue` is the work-queue counter the launch's warps pull items from (zero
// before the launch): the context's own for rm_render_batch, the static
// scratch's for the allocation-free entry point.
void launch_render_batch(Ctx& c, ViewDev* views_dev, int n, int64_t total_items, const rm_launch& L,
                         unsigned long long* queue, unsigned long long* counters) {
  BatchArgs a;
  a.views = views_dev;
  a.nviews = n;
  a.total_items = total_items;
  a.tile_w = L.tile_w;
  a.tile_h = L.tile_h;
  a.rpl = L.rays_per_lane;
  int grid = c.sm_count * (L.ctas_per_sm > 0 ? L.ctas_per_sm : 4);
  MarchParams mp = march_params(c);
  auto go = [&](auto kern) {
    kern<<<grid, 32 * WARPS_PER_CTA, 0, c.stream>>>(c.index(), a, mp, queue, counters);
  };
  const int cps = L.ctas_per_sm;
  if (mp.search == 1) {
    if (cps >= 8) go(k_march_batch<8>);
    else if (cps >= 7) go(k_march_batch<7>);
    else if (cps >= 6) go(k_march_batch<6>);
    else if (cps >= 5) go(k_march_batch<5>);
    else go(k_march_batch<4>);
  } else {
    go(k_march_batch_lane);
  }
}

}  // namespace rm
