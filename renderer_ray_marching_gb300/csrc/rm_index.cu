// rm_index.cu -- device-built spatial index replacing the FLANN CUDA kd-tree
// (third_party/flann/algorithms/kdtree_cuda_builder.h:483-599, which sorts
// x, y and z separately and syncs with the host once per tree level).
//
// Build, all on the device with no host round trip between passes:
//   1. bounds:   block-reduced min/max of the cloud (+ a non-finite flag);
//   2. morton:   30-bit Morton key of each point, quantised per axis;
//   3. sort:     LSD radix sort of (key, cloud index), 4 passes of 8 bits,
//                stable warp-level ranking with __match_any_sync;
//   4. gather:   packed float4 records (x, y, z, radius) and colours in key
//                order, plus the sorted<->cloud index maps;
//   5. tree:     fixed-size leaves of `leaf` consecutive records; an
//                implicit 4-ary tree over them whose nodes store their four
//                children's boxes as one 128-byte group (min x/y/z, max
//                x/y/z as float4 lanes), built bottom-up one level per launch.
// The kNN answers do not depend on the build order: searches are exact with
// (d2, cloud index) ordering, so only speed depends on the layout.
#include "rm_internal.h"

#include <cstring>

namespace rm {

// ---------------------------------------------------------------- bounds
__global__ void k_pack_points(const float* __restrict__ xyz, int stride, int64_t n,
                              float4* __restrict__ pos) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float* p = xyz + i * stride;
    pos[i] = make_float4(p[0], p[1], p[2], 0.0f);
  }
}

__global__ void k_pack_colours(const uint8_t* __restrict__ rgb, int64_t n,
                               uint32_t* __restrict__ packed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t r = rgb ? rgb[3 * i + 0] : 255u;
    uint32_t g = rgb ? rgb[3 * i + 1] : 255u;
    uint32_t b = rgb ? rgb[3 * i + 2] : 255u;
    packed[i] = r | (g << 8) | (b << 16);
  }
}

// Per-block partial bounds: out[block * 8 + {0..5}] = lo xyz, hi xyz;
// [6] = 1 if a non-finite coordinate was seen.
__global__ void k_bounds_partial(const float4* __restrict__ pos, int64_t n,
                                 float* __restrict__ out) {
  float lo[3] = {INFINITY, INFINITY, INFINITY};
  float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  float bad = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 p = pos[i];
    float c[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (!isfinite(c[a])) bad = 1.0f;
      lo[a] = fminf(lo[a], c[a]);
      hi[a] = fmaxf(hi[a], c[a]);
    }
  }
  __shared__ float sh[7][32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
      hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
    }
    bad = fmaxf(bad, __shfl_xor_sync(0xffffffffu, bad, off));
  }
  if (lane == 0) {
    for (int a = 0; a < 3; ++a) {
      sh[a][warp] = lo[a];
      sh[3 + a][warp] = hi[a];
    }
    sh[6][warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    int nw = blockDim.x >> 5;
    float v = sh[threadIdx.x][0];
    for (int w = 1; w < nw; ++w) {
      float x = sh[threadIdx.x][w];
      v = (threadIdx.x < 3) ? fminf(v, x) : fmaxf(v, x);
    }
    out[blockIdx.x * 8 + threadIdx.x] = v;
  }
}

__global__ void k_bounds_final(const float* __restrict__ part, int nblocks,
                               float* __restrict__ out) {
  int a = threadIdx.x;
  if (a >= 7) return;
  float v = part[a];
  for (int b = 1; b < nblocks; ++b) {
    float x = part[b * 8 + a];
    v = (a < 3) ? fminf(v, x) : fmaxf(v, x);
  }
  out[a] = v;
}

// ---------------------------------------------------------------- morton
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_morton(const float4* __restrict__ pos, int64_t n, const float* __restrict__ bounds,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  float lx = bounds[0], ly = bounds[1], lz = bounds[2];
  float sx = 1023.0f / fmaxf(bounds[3] - lx, 1e-30f);
  float sy = 1023.0f / fmaxf(bounds[4] - ly, 1e-30f);
  float sz = 1023.0f / fmaxf(bounds[5] - lz, 1e-30f);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 p = pos[i];
    uint32_t qx = (uint32_t)fminf(fmaxf((p.x - lx) * sx, 0.0f), 1023.0f);
    uint32_t qy = (uint32_t)fminf(fmaxf((p.y - ly) * sy, 0.0f), 1023.0f);
    uint32_t qz = (uint32_t)fminf(fmaxf((p.z - lz) * sz, 0.0f), 1023.0f);
    keys[i] = (spread10(qx) << 2) | (spread10(qy) << 1) | spread10(qz);
    vals[i] = (uint32_t)i;
  }
}

// ---------------------------------------------------------------- radix sort
// Tile = SORT_THREADS threads x SORT_ITEMS keys; warp w owns the contiguous
// run [w*32*SORT_ITEMS, (w+1)*32*SORT_ITEMS) of its tile, processed in
// rounds of 32 consecutive keys, so ranks follow input order (stable).
constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 16;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int RADIX = 256;

__global__ void __launch_bounds__(SORT_THREADS)
k_sort_hist(const uint32_t* __restrict__ keys, int64_t n, int shift, int64_t ntiles,
            uint32_t* __restrict__ counts) {
  __shared__ uint32_t hist[RADIX];
  for (int d = threadIdx.x; d < RADIX; d += blockDim.x) hist[d] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * SORT_TILE;
  for (int k = threadIdx.x; k < SORT_TILE; k += SORT_THREADS) {
    int64_t i = base + k;
    if (i < n) atomicAdd(&hist[(keys[i] >> shift) & (RADIX - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += blockDim.x)
    counts[(int64_t)d * ntiles + blockIdx.x] = hist[d];
}

// Exclusive scan of `len` uint32 in place, block level: each block scans
// SCAN_TILE elements and writes its total.
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int nw = blockDim.x >> 5;
    uint32_t s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= off) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  uint32_t prefix = warp > 0 ? warp_sums[warp - 1] : 0u;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return prefix + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_tiles(uint32_t* __restrict__ data, int64_t len, uint32_t* __restrict__ tile_sums) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = (base + k < len) ? data[base + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, &total);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    if (base + k < len) data[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Single block: exclusive scan of the tile sums (any length).
__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_sums(uint32_t* __restrict__ sums, int64_t len) {
  uint32_t carry = 0;
  for (int64_t start = 0; start < len; start += SCAN_THREADS) {
    int64_t i = start + threadIdx.x;
    uint32_t v = i < len ? sums[i] : 0u;
    uint32_t total;
    uint32_t ex = block_exclusive_scan(v, &total);
    if (i < len) sums[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_add(uint32_t* __restrict__ data, int64_t len, const uint32_t* __restrict__ tile_sums) {
  uint32_t add = tile_sums[blockIdx.x];
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS) {
    int64_t i = base + k;
    if (i < len) data[i] += add;
  }
}

__global__ void __launch_bounds__(SORT_THREADS)
k_sort_scatter(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
               int64_t n, int shift, int64_t ntiles, const uint32_t* __restrict__ offsets,
               uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t wcnt[SORT_WARPS][RADIX];
  __shared__ uint32_t gbase[RADIX];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = lane; d < RADIX; d += 32) wcnt[warp][d] = 0;
  for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS)
    gbase[d] = offsets[(int64_t)d * ntiles + blockIdx.x];
  __syncthreads();
  const uint32_t lt_mask = (1u << lane) - 1u;
  int64_t wbase = (int64_t)blockIdx.x * SORT_TILE + (int64_t)warp * 32 * SORT_ITEMS;
  uint32_t key[SORT_ITEMS], val[SORT_ITEMS], rank[SORT_ITEMS];
#pragma unroll
  for (int r = 0; r < SORT_ITEMS; ++r) {
    int64_t i = wbase + r * 32 + lane;
    bool valid = i < n;
    key[r] = valid ? keys_in[i] : 0u;
    val[r] = valid ? vals_in[i] : 0u;
    // invalid lanes use a private digit value RADIX that matches no real digit
    uint32_t dig = valid ? ((key[r] >> shift) & (RADIX - 1)) : (uint32_t)RADIX;
    uint32_t peers = __match_any_sync(0xffffffffu, dig);
    uint32_t before = __popc(peers & lt_mask);
    uint32_t prev = valid ? wcnt[warp][dig] : 0u;
    __syncwarp();
    if (valid && before == 0) wcnt[warp][dig] = prev + __popc(peers);
    __syncwarp();
    rank[r] = prev + before;
  }
  __syncthreads();
  // per digit: exclusive prefix over warps
  for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; ++w) {
      uint32_t c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < SORT_ITEMS; ++r) {
    int64_t i = wbase + r * 32 + lane;
    if (i < n) {
      uint32_t dig = (key[r] >> shift) & (RADIX - 1);
      uint32_t dst = gbase[dig] + wcnt[warp][dig] + rank[r];
      keys_out[dst] = key[r];
      vals_out[dst] = val[r];
    }
  }
}

// ---------------------------------------------------------------- gather
__global__ void k_gather(const float4* __restrict__ pos, const uint32_t* __restrict__ packed_rgb,
                         const float* __restrict__ radii_clamped, const uint32_t* __restrict__ order,
                         int64_t n, float4* __restrict__ rec, float4* __restrict__ col,
                         int32_t* __restrict__ perm, int32_t* __restrict__ iperm) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    uint32_t i = order[s];
    float4 p = pos[i];
    float r = radii_clamped ? radii_clamped[i] : 0.0f;
    rec[s] = make_float4(p.x, p.y, p.z, r);
    uint32_t c = packed_rgb[i];
    // uint8 / 255.0f as the PLY loader does (src/pointcloud.cpp:55)
    col[s] = make_float4(__fdiv_rn((float)(c & 255u), 255.0f),
                         __fdiv_rn((float)((c >> 8) & 255u), 255.0f),
                         __fdiv_rn((float)((c >> 16) & 255u), 255.0f), 1.0f);
    perm[s] = (int32_t)i;
    iperm[i] = (int32_t)s;
  }
}

// ---------------------------------------------------------------- tree
// Leaf slot l (level `depth`) -> lane (l & 3) of group (l >> 2) of level depth-1.
__global__ void k_leaf_boxes(const float4* __restrict__ rec, int64_t n, int leaf, int depth,
                             int64_t nslots, float4* __restrict__ groups) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nslots;
       l += (int64_t)gridDim.x * blockDim.x) {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    int64_t start = l * leaf;
    int64_t end = min(start + leaf, n);
    for (int64_t i = start; i < end; ++i) {
      float4 p = rec[i];
      lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
      hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
    float* g = reinterpret_cast<float*>(groups + (size_t)GROUP_F4 * (size_t)(group_offset(depth - 1) + (l >> 2)));
    int c = (int)(l & 3);
    g[0 * 4 + c] = lo[0]; g[1 * 4 + c] = lo[1]; g[2 * 4 + c] = lo[2];
    g[3 * 4 + c] = hi[0]; g[4 * 4 + c] = hi[1]; g[5 * 4 + c] = hi[2];
    if (c == 0) {
      g[24] = g[25] = g[26] = g[27] = 0.0f;
      g[28] = g[29] = g[30] = g[31] = 0.0f;
    }
  }
}

// Node j of level lvl (1 <= lvl < depth): union of its group -> lane of its parent's group.
__global__ void k_level_up(int lvl, float4* __restrict__ groups) {
  int64_t count = 1ll << (2 * lvl);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count;
       j += (int64_t)gridDim.x * blockDim.x) {
    const float4* g = groups + (size_t)GROUP_F4 * (size_t)(group_offset(lvl) + j);
    float4 lx = g[0], ly = g[1], lz = g[2], hx = g[3], hy = g[4], hz = g[5];
    float lo0 = fminf(fminf(lx.x, lx.y), fminf(lx.z, lx.w));
    float lo1 = fminf(fminf(ly.x, ly.y), fminf(ly.z, ly.w));
    float lo2 = fminf(fminf(lz.x, lz.y), fminf(lz.z, lz.w));
    float hi0 = fmaxf(fmaxf(hx.x, hx.y), fmaxf(hx.z, hx.w));
    float hi1 = fmaxf(fmaxf(hy.x, hy.y), fmaxf(hy.z, hy.w));
    float hi2 = fmaxf(fmaxf(hz.x, hz.y), fmaxf(hz.z, hz.w));
    float* p = reinterpret_cast<float*>(groups + (size_t)GROUP_F4 * (size_t)(group_offset(lvl - 1) + (j >> 2)));
    int c = (int)(j & 3);
    p[0 * 4 + c] = lo0; p[1 * 4 + c] = lo1; p[2 * 4 + c] = lo2;
    p[3 * 4 + c] = hi0; p[4 * 4 + c] = hi1; p[5 * 4 + c] = hi2;
    if (c == 0) {
      p[24] = p[25] = p[26] = p[27] = 0.0f;
      p[28] = p[29] = p[30] = p[31] = 0.0f;
    }
  }
}

__global__ void k_set_radius(float4* __restrict__ rec, const int32_t* __restrict__ perm,
                             const float* __restrict__ radii_clamped, int64_t n) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x)
    rec[s].w = radii_clamped[perm[s]];
}

__global__ void k_clamp_radii(const float* __restrict__ in, int64_t n, float max_radius,
                              float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float r = in[i];
    // main.cu:144-149
    out[i] = (max_radius > 0.0f && r > max_radius) ? max_radius : r;
  }
}

// Maximum radius (for the culling bound); radii are >= 0 so the float bit
// pattern orders like an unsigned integer.
__global__ void k_max_radius(const float* __restrict__ r, int64_t n, unsigned int* __restrict__ out) {
  float m = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, r[i]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// ---------------------------------------------------------------- host side
static int grid_for(int64_t n, int threads, int max_blocks = 152 * 32) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return (int)b;
}

void launch_pack_points(Ctx& c, const float* xyz, int stride, int64_t n) {
  k_pack_points<<<grid_for(n, 256), 256, 0, c.stream>>>(xyz, stride, n, c.pos.ptr<float4>());
}

void launch_pack_colours(Ctx& c, const uint8_t* rgb, int64_t n) {
  k_pack_colours<<<grid_for(n, 256), 256, 0, c.stream>>>(rgb, n, c.rgb.ptr<uint32_t>());
}

void launch_clamp_radii_only(Ctx& c, const float* in, float max_radius) {
  k_clamp_radii<<<grid_for(c.n, 256), 256, 0, c.stream>>>(in, c.n, max_radius,
                                                            c.radii_clamped.ptr<float>());
}

void launch_set_radius(Ctx& c) {
  k_set_radius<<<grid_for(c.n, 256), 256, 0, c.stream>>>(c.rec.ptr<float4>(), c.perm.ptr<int32_t>(),
                                                          c.radii_clamped.ptr<float>(), c.n);
}

void launch_clamp_radii(Ctx& c, const float* in, float max_radius) {
  launch_clamp_radii_only(c, in, max_radius);
  launch_set_radius(c);
  refresh_max_radius(c);
}

void refresh_max_radius(Ctx& c) {
  unsigned int* mr = c.scalars.ptr<unsigned int>() + 8;
  CK(cudaMemsetAsync(mr, 0, sizeof(unsigned int), c.stream));
  k_max_radius<<<grid_for(c.n, 256, 1024), 256, 0, c.stream>>>(c.radii_clamped.ptr<float>(), c.n, mr);
  unsigned int bits = 0;
  CK(cudaMemcpyAsync(&bits, mr, sizeof(bits), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  float r;
  memcpy(&r, &bits, sizeof(r));
  c.max_r = (r < INFINITY) ? r : INFINITY;
}

// Builds the index from c.pos / c.rgb.  Returns false (with c.err set) on
// invalid input.
bool build_index(Ctx& c) {
  const int64_t n = c.n;
  cudaStream_t st = c.stream;
  // bounds
  int nb = grid_for(n, 256, 1024);
  c.scratch_bounds.reserve((size_t)nb * 8 * sizeof(float));
  k_bounds_partial<<<nb, 256, 0, st>>>(c.pos.ptr<float4>(), n, c.scratch_bounds.ptr<float>());
  k_bounds_final<<<1, 32, 0, st>>>(c.scratch_bounds.ptr<float>(), nb, c.scalars.ptr<float>());
  float hb[8];
  CK(cudaMemcpyAsync(hb, c.scalars.ptr<float>(), 8 * sizeof(float), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (hb[6] != 0.0f) {
    c.err = "cloud contains non-finite coordinates";
    return false;
  }
  for (int a = 0; a < 6; ++a) c.bounds[a] = hb[a];

  // keys
  c.keys[0].reserve((size_t)n * 4);
  c.keys[1].reserve((size_t)n * 4);
  c.vals[0].reserve((size_t)n * 4);
  c.vals[1].reserve((size_t)n * 4);
  k_morton<<<grid_for(n, 256), 256, 0, st>>>(c.pos.ptr<float4>(), n, c.scalars.ptr<float>(),
                                              c.keys[0].ptr<uint32_t>(), c.vals[0].ptr<uint32_t>());
  // radix sort, 30-bit keys: shifts 0, 8, 16, 24
  int64_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
  int64_t clen = ntiles * RADIX;
  int64_t nscan = (clen + SCAN_TILE - 1) / SCAN_TILE;
  c.sort_counts.reserve((size_t)clen * 4);
  c.scan_sums.reserve((size_t)(nscan + 1) * 4);
  int cur = 0;
  for (int shift = 0; shift < 30; shift += 8) {
    uint32_t* cnt = c.sort_counts.ptr<uint32_t>();
    k_sort_hist<<<(unsigned)ntiles, SORT_THREADS, 0, st>>>(c.keys[cur].ptr<uint32_t>(), n, shift, ntiles, cnt);
    k_scan_tiles<<<(unsigned)nscan, SCAN_THREADS, 0, st>>>(cnt, clen, c.scan_sums.ptr<uint32_t>());
    k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(c.scan_sums.ptr<uint32_t>(), nscan);
    k_scan_add<<<(unsigned)nscan, SCAN_THREADS, 0, st>>>(cnt, clen, c.scan_sums.ptr<uint32_t>());
    k_sort_scatter<<<(unsigned)ntiles, SORT_THREADS, 0, st>>>(
        c.keys[cur].ptr<uint32_t>(), c.vals[cur].ptr<uint32_t>(), n, shift, ntiles, cnt,
        c.keys[cur ^ 1].ptr<uint32_t>(), c.vals[cur ^ 1].ptr<uint32_t>());
    cur ^= 1;
  }
  // gather
  c.rec.reserve((size_t)n * sizeof(float4));
  c.col.reserve((size_t)n * sizeof(float4));
  c.perm.reserve((size_t)n * 4);
  c.iperm.reserve((size_t)n * 4);
  k_gather<<<grid_for(n, 256), 256, 0, st>>>(
      c.pos.ptr<float4>(), c.rgb.ptr<uint32_t>(), c.have_radii ? c.radii_clamped.ptr<float>() : nullptr,
      c.vals[cur].ptr<uint32_t>(), n, c.rec.ptr<float4>(), c.col.ptr<float4>(), c.perm.ptr<int32_t>(),
      c.iperm.ptr<int32_t>());
  // tree
  int leaf = c.cfg.leaf_size;
  int64_t nleaves = (n + leaf - 1) / leaf;
  int depth = 1;
  while ((1ll << (2 * depth)) < nleaves) ++depth;
  if (depth > MAX_LEVELS) {
    c.err = "cloud too large for the index depth limit";
    return false;
  }
  int64_t ngroups = group_offset(depth);
  c.groups.reserve((size_t)ngroups * GROUP_F4 * sizeof(float4));
  int64_t nslots = 1ll << (2 * depth);
  k_leaf_boxes<<<grid_for(nslots, 256), 256, 0, st>>>(c.rec.ptr<float4>(), n, leaf, depth, nslots,
                                                       c.groups.ptr<float4>());
  for (int lvl = depth - 1; lvl >= 1; --lvl)
    k_level_up<<<grid_for(1ll << (2 * lvl), 256), 256, 0, st>>>(lvl, c.groups.ptr<float4>());
  c.depth = depth;
  c.nleaves = nleaves;
  CK(cudaGetLastError());
  if (c.have_radii) refresh_max_radius(c);
  c.have_index = true;
  return true;
}

}  // namespace rm
