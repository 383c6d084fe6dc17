// rm_radii.cu -- exact nearest-neighbour radii and the general kNN query.
//
// Replaces the reference's radii precompute (main.cu:107-113): FLANN
// nearestKernel with k = 2 (kdtree_cuda_3d_index.cu:132-154, one thread per
// query, result arrays in global memory), followed by a host loop doing 2N
// synchronous device_reference copies for sqrt, and a separate clamp pass
// (main.cu:144-149).  Here one kernel does search, sqrt, clamp and the
// scatter back to cloud order.  Threads walk the points in index (Morton)
// order, so the 32 queries of a warp are spatial neighbours and their tree
// walks touch the same groups and leaves (L1/L2 hits).
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
// point itself and its next (or previous) record, and walks the tree once
// for all 32 (packet_knn).  Same results as k_radii.
constexpr int RADII_WARPS = 4;
__global__ void __launch_bounds__(32 * RADII_WARPS)
k_radii_packet(IndexDev ix, float max_radius, float* __restrict__ radii_out, int32_t* __restrict__ nn_out,
               float* __restrict__ radii_clamped, unsigned long long* __restrict__ err) {
  __shared__ PacketStack stacks[RADII_WARPS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nwarps = (int64_t)gridDim.x * RADII_WARPS;
  unsigned leaves = 0, nodes = 0;
  for (int64_t wbase = ((int64_t)blockIdx.x * RADII_WARPS + warp) * 32; wbase < ix.n; wbase += nwarps * 32) {
    const int64_t s = wbase + lane;
    const bool active = s < ix.n;
    float4 q = active ? __ldg(ix.rec + s) : make_float4(0.f, 0.f, 0.f, 0.f);
    KList<2> L;
    klist_init<2>(L);
    if (active) {
      klist_insert<2>(L, d2_point(q, q.x, q.y, q.z), (int32_t)s, q.w, ix.perm);
      int64_t nb = (s + 1 < ix.n) ? s + 1 : s - 1;
      if (nb >= 0 && nb != s) {
        float4 c = __ldg(ix.rec + nb);
        klist_insert<2>(L, d2_point(c, q.x, q.y, q.z), (int32_t)nb, c.w, ix.perm);
      }
    }
    if (!packet_knn(ix, active, q.x, q.y, q.z, L, stacks[warp], leaves, nodes) && active) atomicAdd(err, 1ull);
    if (active) {
      float r = __fsqrt_rn(L.d[1]);
      int32_t i = __ldg(ix.perm + s);
      if (radii_out) radii_out[i] = r;
      if (nn_out) nn_out[i] = L.s[1] >= 0 ? __ldg(ix.perm + L.s[1]) : -1;
      radii_clamped[i] = (max_radius > 0.0f && r > max_radius) ? max_radius : r;
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

void launch_radii(Ctx& c, float max_radius, float* radii_out, int32_t* nn_out) {
  unsigned long long* err = c.scalars.ptr<unsigned long long>() + 8;
  if (c.launch.search == 1) {
    k_radii_packet<<<blocks_for(c, c.n, 32 * RADII_WARPS), 32 * RADII_WARPS, 0, c.stream>>>(
        c.index(), max_radius, radii_out, nn_out, c.radii_clamped.ptr<float>(), err);
  } else {
    k_radii<<<blocks_for(c, c.n, 128), 128, 0, c.stream>>>(c.index(), max_radius, radii_out, nn_out,
                                                           c.radii_clamped.ptr<float>(), err);
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
