// rm_march.cu -- the sphere-tracing marcher (replaces the reference's
// render kernel, src/ray_marching.cu:63-91, and its per-step FLANN query,
// :202-292).
//
// Work unit: one warp marches the rays of a screen tile (tile_w x tile_h
// pixels, 32 rays; with rays_per_lane > 1 an item is rays_per_lane such
// tiles stacked vertically and a lane whose ray ends takes the item's next
// pixel).  Each distance step is an exact 10-NN of the step position:
//
//   1. seed: every lane re-measures its previous step's 10 points at the new
//      position (valid candidates, so its k-th distance is finite at once);
//   2. cooperative gather: lanes whose seeded ball (radius = sqrt of the
//      seeded 10th distance) is small form a group; the warp takes the box Q
//      holding all their balls and walks the tree once, 32 nodes per round,
//      collecting every leaf whose box meets Q;
//   3. staged scan: the warp copies those leaves' records into shared memory
//      with coalesced loads and every lane of the group tests every staged
//      point (shared-memory broadcast reads).  Every point inside a lane's
//      ball lies in Q, hence in a collected leaf, so the lane's 10-NN is
//      exact;
//   4. lanes outside the group (first step, empty space), or all lanes when
//      the gather exceeds its capacity, run the per-lane tree search.
// Then the step value min(sqrtf(d2) - r) and the reference's termination
// tests (MIN_DIST hit, far plane, MAX_STEPS).
//
// Plain form (rm_render): one warp per 8x4 tile, four warps per CTA.
// Batched form (rm_render_batch): a persistent kernel whose warps pull items
// of any view from one global counter; the whole launch is a CUDA graph.
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

// Per-warp shared memory of the cooperative step.
constexpr int WARPS_PER_CTA = 4;
constexpr int FRONTIER_CAP = 128;   // nodes per tree level
constexpr int LEAF_CAP = 128;       // leaves per gather
constexpr int STAGE_CAP = 256;      // staged records per scan round

struct WarpSmem {
  uint32_t front[2][FRONTIER_CAP];
  uint32_t leaves[LEAF_CAP];
  float4 rec[STAGE_CAP];
  int32_t pos[STAGE_CAP];
};

struct MarchParams {
  ClipBox clip;
  float coop_r2;  // lanes whose seeded 10th distance (squared) is at most this join the gather
};

// View as seen by the marcher.
struct ViewArgs {
  const float* m;
  int32_t width, height;
  float pane;
  float4* rgbd;
  int32_t* hit;
  float* depth;
  int32_t* steps;
};

// counters: [0] steps, [1] rays, [2] hits, [3] search errors,
//           [4] gathered lane-steps, [5] per-lane lane-steps, [6] gather overflows
struct LaneCounters {
  unsigned long long steps = 0, rays = 0, hits = 0, bad = 0, coop = 0, solo = 0, overflow = 0;
};

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

// Collects every leaf whose box meets Q into sm.leaves.  Returns the leaf
// count, or -1 when a level or the leaf list exceeds its capacity.  All 32
// lanes call it with the same Q.
__device__ int gather_leaves(const IndexDev& ix, const float qlo[3], const float qhi[3], WarpSmem& sm) {
  const int lane = threadIdx.x & 31;
  int cur = 0;
  int count = 1;
  if (lane == 0) sm.front[0][0] = 0u;
  __syncwarp();
  for (int lvl = 0; lvl < ix.depth; ++lvl) {
    const bool last = (lvl + 1 == ix.depth);
    uint32_t* out = last ? sm.leaves : sm.front[cur ^ 1];
    const int cap = last ? LEAF_CAP : FRONTIER_CAP;
    int ncount = 0;
    for (int b = 0; b < count; b += 32) {
      int i = b + lane;
      unsigned m4 = 0;
      uint32_t j = 0;
      if (i < count) {
        j = sm.front[cur][i];
        const float4* g = ix.groups + (size_t)GROUP_F4 * (size_t)(group_offset(lvl) + j);
        float4 lx = __ldg(g + 0), ly = __ldg(g + 1), lz = __ldg(g + 2);
        float4 hx = __ldg(g + 3), hy = __ldg(g + 4), hz = __ldg(g + 5);
        float alx[4] = {lx.x, lx.y, lx.z, lx.w}, aly[4] = {ly.x, ly.y, ly.z, ly.w}, alz[4] = {lz.x, lz.y, lz.z, lz.w};
        float ahx[4] = {hx.x, hx.y, hx.z, hx.w}, ahy[4] = {hy.x, hy.y, hy.z, hy.w}, ahz[4] = {hz.x, hz.y, hz.z, hz.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          bool meet = alx[c] <= qhi[0] && ahx[c] >= qlo[0] && aly[c] <= qhi[1] && ahy[c] >= qlo[1] &&
                      alz[c] <= qhi[2] && ahz[c] >= qlo[2];
          m4 |= meet ? (1u << c) : 0u;
        }
      }
      int n = __popc(m4);
      int incl = n;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
      }
      int total = __shfl_sync(0xffffffffu, incl, 31);
      if (ncount + total > cap) return -1;
      int w = ncount + incl - n;
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (m4 & (1u << c)) out[w++] = j * 4u + (uint32_t)c;
      ncount += total;
    }
    __syncwarp();
    if (last) return ncount;
    if (ncount == 0) return 0;
    cur ^= 1;
    count = ncount;
  }
  return 0;
}

// Stages the records of the gathered leaves and lets every `member` lane
// consider every staged point.  All lanes call it.
__device__ void scan_gathered(const IndexDev& ix, WarpSmem& sm, int nleaves, bool member, float px,
                              float py, float pz, KSet& L) {
  const int lane = threadIdx.x & 31;
  const int leaf = ix.leaf;
  const int per_round = STAGE_CAP / leaf;  // whole leaves per staging round
  for (int l0 = 0; l0 < nleaves; l0 += per_round) {
    int nl = min(per_round, nleaves - l0);
    int slots = nl * leaf;
    __syncwarp();
    for (int k = lane; k < slots; k += 32) {
      int li = k / leaf, o = k - li * leaf;
      int64_t p = (int64_t)sm.leaves[l0 + li] * leaf + o;
      if (p < ix.n) {
        sm.rec[k] = __ldg(ix.rec + p);
        sm.pos[k] = (int32_t)p;
      } else {
        sm.rec[k] = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
        sm.pos[k] = -1;
      }
    }
    __syncwarp();
    if (member) {
      for (int k = 0; k < slots; ++k) {
        float4 c = sm.rec[k];
        float d = d2_point(c, px, py, pz);
        if (d <= L.wd && sm.pos[k] >= 0) L.consider(d, sm.pos[k], c.w, ix.perm);
      }
    }
  }
  __syncwarp();
}

__device__ __forceinline__ void write_result(const IndexDev& ix, const ViewArgs& v, int64_t pix, int32_t s,
                                             float depth, int32_t steps) {
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
// of view v.  All 32 lanes call it.
__device__ void march_item(const IndexDev& ix, const ViewArgs& v, int x0, int y0, int tile_w,
                           int tile_h, int rpl, const MarchParams& mp, WarpSmem& sm, LaneCounters& cnt) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int item_rays = tile_w * tile_h * rpl;
  int next = 0;
  bool has = false;
  int64_t pix = 0;
  Ray r;
  float t = 0.0f, t_stop = 0.0f;
  int nsteps = 0;
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
          pix = (int64_t)y * v.width + x;
          r = make_ray(v.m, v.width, v.height, v.pane, x, y);
          t_stop = clip_exit(r, mp.clip);
          t = r.t_near;
          nsteps = 0;
          L.clear();
        }
      }
      next += __popc(need);
      need = __ballot_sync(FULL, !has);
    }
    if (__ballot_sync(FULL, has) == 0) break;

    bool stepping = has && !(t > t_stop);  // past the exit bound: a miss (culled)
    if (has && !stepping) {
      write_result(ix, v, pix, -1, 0.0f, nsteps);
      cnt.steps += nsteps;
      cnt.rays += 1;
      has = false;
    }
    float px = __fmaf_rn(r.dx, t, r.ox);
    float py = __fmaf_rn(r.dy, t, r.oy);
    float pz = __fmaf_rn(r.dz, t, r.oz);
    if (stepping) L.rewarm(ix, px, py, pz);
    bool member = stepping && L.wd <= mp.coop_r2;
    unsigned mm = __ballot_sync(FULL, member);
    bool done = false;
    if (__popc(mm) >= 2) {
      // Q: box of the members' balls; the radius is rounded outwards so that
      // every point whose computed d2 is <= wd lies inside
      float rad = member ? __fmul_rn(__fsqrt_rn(L.wd), 1.0f + 1e-5f) + 1e-5f : 0.0f;
      float qlo[3], qhi[3];
      qlo[0] = warp_min(member ? px - rad : INFINITY);
      qlo[1] = warp_min(member ? py - rad : INFINITY);
      qlo[2] = warp_min(member ? pz - rad : INFINITY);
      qhi[0] = warp_max(member ? px + rad : -INFINITY);
      qhi[1] = warp_max(member ? py + rad : -INFINITY);
      qhi[2] = warp_max(member ? pz + rad : -INFINITY);
      int nl = gather_leaves(ix, qlo, qhi, sm);
      if (nl >= 0) {
        scan_gathered(ix, sm, nl, member, px, py, pz, L);
        done = member;
      } else {
        cnt.overflow += (lane == 0) ? 1 : 0;
      }
    }
    if (stepping) {
      if (!done) {
        if (!knn_search(ix, px, py, pz, L)) cnt.bad += 1;
        cnt.solo += 1;
      } else {
        cnt.coop += 1;
      }
      int32_t s;
      float step = L.step_value(ix.perm, &s);
      ++nsteps;
      t = __fadd_rn(t, step);
      bool fin = false;
      int32_t hs = -1;
      float hd = 0.0f;
      if (step < MIN_DIST) {  // src/ray_marching.cu:219-222
        fin = true;
        hs = s;
        hd = t;
      } else if (t > r.t_far || nsteps >= MAX_STEPS) {
        fin = true;
      }
      if (fin) {
        write_result(ix, v, pix, hs, hd, nsteps);
        cnt.steps += nsteps;
        cnt.rays += 1;
        cnt.hits += hs >= 0 ? 1 : 0;
        has = false;
      }
    }
  }
}

__device__ __forceinline__ void flush_counters(LaneCounters& c, unsigned long long* counters) {
  unsigned long long v[7] = {c.steps, c.rays, c.hits, c.bad, c.coop, c.solo, c.overflow};
#pragma unroll
  for (int k = 0; k < 7; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 7; ++k)
      if (v[k]) atomicAdd(counters + k, v[k]);
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
__global__ void __launch_bounds__(32 * WARPS_PER_CTA)
k_march_plain(IndexDev ix, PlainArgs a, MarchParams mp, unsigned long long* __restrict__ counters) {
  __shared__ WarpSmem smem[WARPS_PER_CTA];
  const int warp = threadIdx.x >> 5;
  int tiles_x = (a.width + 7) / 8;
  int tile = blockIdx.x * WARPS_PER_CTA + warp;
  int tiles = tiles_x * ((a.height + 3) / 4);
  LaneCounters cnt;
  if (tile < tiles) {
    ViewArgs v;
    v.m = a.m;
    v.width = a.width;
    v.height = a.height;
    v.pane = view_pane(a.width, a.fov);
    v.rgbd = a.rgbd;
    v.hit = a.hit;
    v.depth = a.depth;
    v.steps = a.steps;
    march_item(ix, v, (tile % tiles_x) * 8, (tile / tiles_x) * 4, 8, 4, 1, mp, smem[warp], cnt);
  }
  flush_counters(cnt, counters);
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

__global__ void __launch_bounds__(32 * WARPS_PER_CTA)
k_march_batch(IndexDev ix, BatchArgs a, MarchParams mp, unsigned long long* __restrict__ queue,
              unsigned long long* __restrict__ counters) {
  __shared__ WarpSmem smem[WARPS_PER_CTA];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  LaneCounters cnt;
  while (true) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(queue, 1ull);
    it = __shfl_sync(0xffffffffu, it, 0);
    if ((int64_t)it >= a.total_items) break;
    int iv = find_view(a.views, a.nviews, (int64_t)it);
    const ViewDev& V = a.views[iv];
    int64_t local = (int64_t)it - V.tile_base;
    ViewArgs v;
    v.m = V.m;
    v.width = V.width;
    v.height = V.height;
    v.pane = V.pane;
    v.rgbd = V.rgbd;
    v.hit = V.hit;
    v.depth = V.depth;
    v.steps = V.steps;
    int x0 = (int)(local % V.tiles_x) * a.tile_w;
    int y0 = (int)(local / V.tiles_x) * (a.tile_h * a.rpl);
    march_item(ix, v, x0, y0, a.tile_w, a.tile_h, a.rpl, mp, smem[warp], cnt);
  }
  flush_counters(cnt, counters);
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
  float cr = c.coop_radius;
  mp.coop_r2 = cr * cr;
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
  k_march_plain<<<grid, 32 * WARPS_PER_CTA, 0, c.stream>>>(c.index(), a, march_params(c), counters);
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
  unsigned long long* queue = c.queue.ptr<unsigned long long>();
  int grid = c.sm_count * (L.ctas_per_sm > 0 ? L.ctas_per_sm : 4);
  k_march_batch<<<grid, 32 * WARPS_PER_CTA, 0, c.stream>>>(c.index(), a, march_params(c), queue, counters);
}

}  // namespace rm
