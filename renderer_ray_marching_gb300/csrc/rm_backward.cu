// rm_backward.cu -- gradient of an image loss through each pixel's first hit.
//
// The reference has no gradient path.  The differentiable model fixed here:
//   colour(p) = colour[hit(p)]                          (float32 RGB)
//   depth(p)  = entry distance of ray p into the sphere (c_hit, r_hit)
// with hit(p) the index stored by the forward pass, held constant.  The
// marcher's own depth stops within MIN_DIST (1e-3) of the union of the
// nearest spheres, so it differs from this analytic surrogate by less than
// MIN_DIST plus one step; the surrogate is what is differentiated.
//
// Per pixel the kernel recomputes the ray exactly as the forward did,
// evaluates t and its gradient in double precision (t = (b - sqrt(disc))/a
// with a = |d|^2, b = d.(c - o), disc = b^2 - a(|c - o|^2 - r^2); the FP64
// evaluation keeps the millimetre-scale discriminant of metre-scale
// operands accurate), scales by the incoming dL/ddepth and accumulates into
// float32 per-point gradients.  Pixels of a warp that share a hit point are
// reduced in registers first (__match_any_sync), so each point receives one
// atomic per warp and channel.
#include "rm_internal.h"

namespace rm {

struct BackArgs {
  const ViewDev* views;
  const int64_t* pix_base;   // per view, first pixel of the view; [n] = total
  int nviews;
  int64_t total;
  const float* dl_drgb;      // 3 floats per pixel
  const float* dl_ddepth;    // 1 float per pixel
  const int32_t* hit;        // cloud index per pixel, -1 = miss
  const int32_t* iperm;      // cloud index -> sorted position
  float* g_rgb;              // 3 floats per point
  float* g_xyz;              // 3 floats per point
  float* g_radius;           // 1 float per point
};

__device__ __forceinline__ int view_of_pixel(const int64_t* base, int n, int64_t p) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_backward(IndexDev ix, BackArgs a) {
  const unsigned FULL = 0xffffffffu;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t first = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // uniform trip count across the warp so every lane reaches the shuffles
  int64_t warp_first = first - (threadIdx.x & 31);
  for (int64_t wbase = warp_first; wbase < a.total; wbase += stride) {
    int64_t p = wbase + (threadIdx.x & 31);
    int32_t h = -1;
    float g[7] = {0, 0, 0, 0, 0, 0, 0};
    if (p < a.total) {
      h = __ldg(a.hit + p);
      if (h >= ix.n) h = -1;  // caller-supplied index outside the cloud: ignored
      if (h >= 0) {
        int v = view_of_pixel(a.pix_base, a.nviews, p);
        const ViewDev& V = a.views[v];
        int64_t local = p - a.pix_base[v];
        int x = (int)(local % V.width), y = (int)(local / V.width);
        Ray r = make_ray(V.m, V.width, V.height, V.pane, x, y);
        int32_t s = __ldg(a.iperm + h);
        float4 c = __ldg(ix.rec + s);
        double d0 = r.dx, d1 = r.dy, d2 = r.dz;
        double oc0 = (double)c.x - (double)r.ox;
        double oc1 = (double)c.y - (double)r.oy;
        double oc2 = (double)c.z - (double)r.oz;
        double rr = c.w;
        double aa = d0 * d0 + d1 * d1 + d2 * d2;
        double b = d0 * oc0 + d1 * oc1 + d2 * oc2;
        double cc = oc0 * oc0 + oc1 * oc1 + oc2 * oc2 - rr * rr;
        double disc = b * b - aa * cc;
        double gc0, gc1, gc2, gr;
        double ia = 1.0 / aa;
        if (disc > 0.0) {
          double is = 1.0 / sqrt(disc);
          gc0 = (d0 - (b * d0 - aa * oc0) * is) * ia;
          gc1 = (d1 - (b * d1 - aa * oc1) * is) * ia;
          gc2 = (d2 - (b * d2 - aa * oc2) * is) * ia;
          gr = -rr * is;
        } else {
          gc0 = d0 * ia;
          gc1 = d1 * ia;
          gc2 = d2 * ia;
          gr = 0.0;
        }
        double ld = (double)__ldg(a.dl_ddepth + p);
        g[0] = __ldg(a.dl_drgb + 3 * p + 0);
        g[1] = __ldg(a.dl_drgb + 3 * p + 1);
        g[2] = __ldg(a.dl_drgb + 3 * p + 2);
        g[3] = (float)(ld * gc0);
        g[4] = (float)(ld * gc1);
        g[5] = (float)(ld * gc2);
        g[6] = (float)(ld * gr);
      }
    }
    unsigned peers = __match_any_sync(FULL, h);
    int leader = __ffs(peers) - 1;
    float sum[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) sum[k] = 0.0f;
    // every lane of the group walks the same peer list, so the masked shuffles line up
    unsigned m = peers;
    while (m) {
      int src = __ffs(m) - 1;
#pragma unroll
      for (int k = 0; k < 7; ++k) sum[k] += __shfl_sync(peers, g[k], src);
      m &= m - 1;
    }
    if (h >= 0 && (int)(threadIdx.x & 31) == leader) {
      atomicAdd(a.g_rgb + 3 * (int64_t)h + 0, sum[0]);
      atomicAdd(a.g_rgb + 3 * (int64_t)h + 1, sum[1]);
      atomicAdd(a.g_rgb + 3 * (int64_t)h + 2, sum[2]);
      atomicAdd(a.g_xyz + 3 * (int64_t)h + 0, sum[3]);
      atomicAdd(a.g_xyz + 3 * (int64_t)h + 1, sum[4]);
      atomicAdd(a.g_xyz + 3 * (int64_t)h + 2, sum[5]);
      atomicAdd(a.g_radius + h, sum[6]);
    }
  }
}

void launch_backward(Ctx& c, const ViewDev* views_dev, int n, int64_t total_pixels,
                     const int64_t* pix_base, const float* dl_drgb, const float* dl_ddepth,
                     const int32_t* hit, float* g_rgb, float* g_xyz, float* g_radius) {
  BackArgs a;
  a.views = views_dev;
  a.pix_base = pix_base;
  a.nviews = n;
  a.total = total_pixels;
  a.dl_drgb = dl_drgb;
  a.dl_ddepth = dl_ddepth;
  a.hit = hit;
  a.iperm = c.iperm.ptr<int32_t>();
  a.g_rgb = g_rgb;
  a.g_xyz = g_xyz;
  a.g_radius = g_radius;
  int64_t blocks = (total_pixels + 255) / 256;
  int64_t cap = (int64_t)c.sm_count * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_backward<<<(unsigned)blocks, 256, 0, c.stream>>>(c.index(), a);
}

}  // namespace rm
