// kset_probe.cu -- test-only probe of the marcher's neighbour set (never
// part of the library).
//
// Runs rm::KSet, the set the marcher keeps its 10 nearest points in, on
// sequences of candidate (d2, sorted position) pairs written by the test:
// one sequence per thread, offered in order with the walk's own filter
// (a candidate is considered only when its d2 is <= the set's current
// bound), starting from placeholders at a given bound as a step does
// (KSet::restart), and read out after KSet::order() as the step value does.
// The sequences are full of exact d2 ties, so the fast insertion, the
// ordered insertion at the set's boundary and the final ordering by cloud
// index are all exercised; the test compares the result with a sort by
// (d2, cloud index) on the host.
#include <cuda_runtime.h>

#include <cstdint>

#include "rm_device.cuh"

namespace {

__global__ void k_kset(const float* __restrict__ d2, const int32_t* __restrict__ pos, const float* __restrict__ bound,
                       const int32_t* __restrict__ perm, int seqs, int len, float* __restrict__ out_d,
                       int32_t* __restrict__ out_s) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= seqs) return;
  rm::KSet L;
#pragma unroll
  for (int j = 0; j < rm::KNN; ++j) {
    L.d[j] = bound[t];
    L.s[j] = -1;
  }
  for (int i = 0; i < len; ++i) {
    const float d = d2[(int64_t)t * len + i];
    const int32_t s = pos[(int64_t)t * len + i];
    if (s >= 0 && d <= L.worst()) L.consider(d, s, perm);
  }
  L.order(perm);
#pragma unroll
  for (int j = 0; j < rm::KNN; ++j) {
    out_d[(int64_t)t * rm::KNN + j] = L.d[j];
    out_s[(int64_t)t * rm::KNN + j] = L.s[j];
  }
}

}  // namespace

// All pointers are device pointers.  d2 and pos: seqs x len candidates
// (pos < 0 pads a sequence); bound: the placeholder bound of each sequence;
// perm: sorted position -> cloud index; out: seqs x 10 entries.
extern "C" int kset_run(const float* d2, const int32_t* pos, const float* bound, const int32_t* perm, int seqs,
                        int len, float* out_d, int32_t* out_s) {
  if (seqs <= 0) return 0;
  k_kset<<<(seqs + 127) / 128, 128>>>(d2, pos, bound, perm, seqs, len, out_d, out_s);
  return (int)cudaDeviceSynchronize();
}
