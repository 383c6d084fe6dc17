// rm_radii.cu -- exact nearest-neighbour radii and the general kNN query.
//
// Replaces the reference's radii precompute (main.cu:107-113): FLANN
// nearestKernel with k = 2 (kdtree_cuda_3d_index.cu:132-154, one thread per
// query, result arrays in global memory), followed by a host loop doing 2N
// synchronous device_reference copies for sqrt, and a separate clamp pass
// (main.cu:144-149).  Here one kernel does the search and the sqrt for every
// point, in index (Morton) order, so the 32 queries of a warp are spatial
// neighbours and their tree walks touch the same groups and leaves (L1/L2
// hits); short passes then write the results in cloud order and clamp.
#include "rm_internal.h"

namespace rm {

__global__ void __launch_bounds__(128)
k_radii(IndexDev ix, float max_radius, float* __restrict__ radii_out, int32_t* __restrict__ nn_out,
        float* __restrict__ radii_clamped, unsigned long long* __restrict__ err) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ix.n;
       s += (int64_t)gridDim.x * blockDim.x) {
    float4 q = __ldg(ix.rec + s);
    KList<2> L;
    klist_init<2>(L);
    if (!knn_search(ix, q.x, q.y, q.z, L)) atomicAdd(err, 1ull);
    // sqrt of the second entry (main.cu:111); +inf when the cloud has one point
    float r = __fsqrt_rn(L.d[1]);
    int32_t i = __ldg(ix.perm + s);
    if (radii_out) radii_out[i] = r;
    if (nn_out) nn_out[i] = L.s[1] >= 0 ? __ldg(ix.perm + L.s[1]) : -1;
    radii_clamped[i] = (max_radius > 0.0f && r > max_radius) ? max_radius : r;
  }
}

// Packet form: a warp takes 32 consecutive sorted points (spatial
// neighbours along the Morton curve), seeds each lane's 2-NN list with the
// point itself and its previous and next records, and walks the tree once
// for all 32 (packet_knn).  Same results as k_radii.
//
// Memory traffic.  Warps take their 32-point chunks from a global counter
// in sorted order, so every resident warp works inside one window of about
// (resident warps x 32) consecutive records -- a few MB, which stays in L2
// while neighbouring warps re-read the same leaves.  (A grid-stride loop
// spreads the resident warps over strides of the whole array, and their
// leaf reads miss L2.)  Results go out in sorted order with coalesced
// stores; k_radii_to_cloud moves them to cloud order afterwards.
constexpr int RADII_WARPS = 4;
__global__ void __launch_bounds__(32 * RADII_WARPS)
k_radii_packet(IndexDev ix, float* __restrict__ r_sorted, int32_t* __restrict__ nn_sorted,
               unsigned long long* __restrict__ next, unsigned long long* __restrict__ err) {
  __shared__ PacketStack stacks[RADII_WARPS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned leaves = 0, nodes = 0;
  while (true) {
    unsigned long long chunk = 0;
    if (lane == 0) chunk = atomicAdd(next, 1ull);
    const int64_t wbase = (int64_t)__shfl_sync(0xffffffffu, chunk, 0) * 32;
    if (wbase >= ix.n) break;
    const int64_t s = wbase + lane;
    const bool active = s < ix.n;
    float4 q = active ? __ldg(ix.rec + s) : make_float4(0.f, 0.f, 0.f, 0.f);
    KList<2> L;
    klist_init<2>(L);
    if (active) {
      // seeds: the point itself and both of its sorted neighbours.  The
      // nearer neighbour bounds the search from its first node; the warp's
      // walk is steered by its loosest lane, and a Morton jump on one side
      // of a point rarely falls on the other (both seeds: -9% at 20M points)
      klist_insert<2>(L, d2_point(q, q.x, q.y, q.z), (int32_t)s, q.w, ix.perm);
      if (s + 1 < ix.n) {
        const float4 c = __ldg(ix.rec + s + 1);
        klist_insert<2>(L, d2_point(c, q.x, q.y, q.z), (int32_t)(s + 1), c.w, ix.perm);
      }
      if (s >= 1) {
        const float4 c = __ldg(ix.rec + s - 1);
        list_consider_unique(L, d2_point(c, q.x, q.y, q.z), (int32_t)(s - 1), c.w, ix.perm);
      }
    }
    if (!packet_knn(ix, active, q.x, q.y, q.z, L, stacks[warp], leaves, nodes) && active) atomicAdd(err, 1ull);
    if (active) {
      // sqrt of the second entry (main.cu:111); +inf when the cloud has one point
      r_sorted[s] = __fsqrt_rn(L.d[1]);
      nn_sorted[s] = L.s[1] >= 0 ? __ldg(ix.perm + L.s[1]) : -1;
    }
  }
}

// Sorted-order radii to cloud order (main.cu:110-113 leaves them in PLY
// order), one output array per launch.  Each launch reads its sorted input
// and perm once, streaming (evict-first), and scatters 4-byte values over
// one array of 4 N bytes; at up to about 25M points that array fits in L2,
// where the scattered stores merge into whole sectors before they reach
// DRAM.  MODE 0: unclamped radius; 1: neighbour's cloud index; 2: radius
// clamped to max_radius (main.cu:144-149) -- the context's render radii --
// also written into the records' .w in sorted order.
template <int MODE>
__global__ void k_radii_to_cloud(const float* __restrict__ r_sorted, const int32_t* __restrict__ nn_sorted,
                                 const int32_t* __restrict__ perm, int64_t n, float max_radius,
                                 void* __restrict__ out, float4* __restrict__ rec) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = __ldcs(perm + s);
    if (MODE == 1) {
      static_cast<int32_t*>(out)[i] = __ldcs(nn_sorted + s);
    } else {
      float r = __ldcs(r_sorted + s);
      if (MODE == 2) {
        r = (max_radius > 0.0f && r > max_radius) ? max_radius : r;
        float4 c = rec[s];  // whole records rewritten: full-sector stores
        c.w = r;
        rec[s] = c;
      }
      static_cast<float*>(out)[i] = r;
    }
  }
}

template <int K>
__global__ void __launch_bounds__(128)
k_knn(IndexDev ix, const float* __restrict__ q, int stride, int64_t m, int k,
      int32_t* __restrict__ idx_out, float* __restrict__ d2_out, unsigned long long* __restrict__ err) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float* p = q + t * stride;
    KList<K> L;
    klist_init<K>(L);
    if (!knn_search(ix, p[0], p[1], p[2], L)) atomicAdd(err, 1ull);
    for (int j = 0; j < k; ++j) {
      int32_t s = L.s[j];
      idx_out[t * k + j] = s >= 0 ? __ldg(ix.perm + s) : -1;
      d2_out[t * k + j] = L.d[j];
    }
  }
}

static int blocks_for(const Ctx& c, int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)c.sm_count * 64;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// Radii of every point: search, then cloud-order outputs, the context's
// clamped radii and the records' radius lanes.
void launch_radii(Ctx& c, float max_radius, float* radii_out, int32_t* nn_out) {
  unsigned long long* err = c.scalars.ptr<unsigned long long>() + 8;
  if (c.launch.search == 1) {
    // sorted-order results in the radix sort's key buffers (N x 4 B each,
    // free once the index is built)
    float* r_sorted = c.keys[0].ptr<float>();
    int32_t* nn_sorted = c.keys[1].ptr<int32_t>();
    unsigned long long* next = c.queue.ptr<unsigned long long>() + 1;
    CK(cudaMemsetAsync(next, 0, sizeof(unsigned long long), c.stream));
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_radii_packet, 32 * RADII_WARPS, 0));
    const int64_t chunks = (c.n + 31) / 32;
    int64_t grid = (int64_t)c.sm_count * (per_sm > 0 ? per_sm : 1);
    const int64_t need = (chunks + RADII_WARPS - 1) / RADII_WARPS;
    if (grid > need) grid = need;
    k_radii_packet<<<(unsigned)grid, 32 * RADII_WARPS, 0, c.stream>>>(c.index(), r_sorted, nn_sorted, next, err);
    const int g = blocks_for(c, c.n, 256);
    const int32_t* perm = c.perm.ptr<int32_t>();
    if (radii_out)
      k_radii_to_cloud<0><<<g, 256, 0, c.stream>>>(r_sorted, nn_sorted, perm, c.n, max_radius, radii_out, nullptr);
    if (nn_out)
      k_radii_to_cloud<1><<<g, 256, 0, c.stream>>>(r_sorted, nn_sorted, perm, c.n, max_radius, nn_out, nullptr);
    k_radii_to_cloud<2><<<g, 256, 0, c.stream>>>(r_sorted, nn_sorted, perm, c.n, max_radius,
                                                 c.radii_clamped.ptr<float>(), c.rec.ptr<float4>());
  } else {
    k_radii<<<blocks_for(c, c.n, 128), 128, 0, c.stream>>>(c.index(), max_radius, radii_out, nn_out,
                                                           c.radii_clamped.ptr<float>(), err);
    launch_set_radius(c);
  }
}

void launch_knn(Ctx& c, const float* q, int stride, int64_t m, int k, int32_t* idx, float* d2) {
  unsigned long long* err = c.scalars.ptr<unsigned long long>() + 8;
  int b = blocks_for(c, m, 128);
  IndexDev ix = c.index();
  if (k <= 2) k_knn<2><<<b, 128, 0, c.stream>>>(ix, q, stride, m, k, idx, d2, err);
  else if (k <= 10) k_knn<10><<<b, 128, 0, c.stream>>>(ix, q, stride, m, k, idx, d2, err);
  else if (k <= 16) k_knn<16><<<b, 128, 0, c.stream>>>(ix, q, stride, m, k, idx, d2, err);
  else k_knn<32><<<b, 128, 0, c.stream>>>(ix, q, stride, m, k, idx, d2, err);
}

}  // namespace rm
