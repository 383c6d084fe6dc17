// fp_contract.cu -- test-only probe of the floating-point contract (never
// part of the library).
//
// The reference's GPU arithmetic is whatever nvcc makes of its source with
// default flags (no fast-math: CMakeLists.txt and cmake/kdtree.cmake set
// none), and nvcc contracts a multiply feeding an add into one fused
// multiply-add.  The library instead writes every rounding step with an
// explicit _rn intrinsic (renderer_ray_marching_gb300/csrc/rm_device.cuh).
// This file evaluates, on the same inputs:
//   - "ref": the reference's source expressions, in the shape they have
//     there, compiled with nvcc's defaults (this file must be built WITHOUT
//     --fmad=false, -use_fast_math or -ftz=true);
//   - "lib": the library's device functions;
// and writes both so that the test can compare their bits.
//
// Expressions restated (shapes only; every helper here is written for this
// probe):
//   FLANN CudaL2::dist, third_party/flann/algorithms/kdtree_cuda_3d_index.cu:186-192:
//       float4 diff = a - b; dot(diff, diff)       (util/cutil_math.h:596-599, 1127-1130;
//       w = 0 on both sides: points are memset to w = 0, the query is (pos, 0))
//   step position, src/ray_marching.cu:216:  ray_origin + ray_dir * t  (float3 ops)
//   plane distances, src/ray_marching.cu:75, 78-79: ZFAR / dot(cam_dir, dir) (float3 dot),
//       cam_dir = -CAMERA_MATRIX[2] with glm's vec4 unary minus (vec4(0) -= v)
//   ray direction, src/ray_marching.cu:71-77: uv = (2 * xy - res) / 2,
//       pane = W / (2 * tanf(0.5 * fov)), dir = normalize(C * vec4(uv, -pane, 0)),
//       with glm 0.9.9.8's published algorithms: mat4 * vec4 as the column sum
//       (c0 x + c1 y) + (c2 z + c3 w), dot(vec4) as (x x' + y y') + (z z' + w w'),
//       normalize(v) = v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
//   step value, src/ray_marching.cu:285:  sqrtf(D) - R
#include <cuda_runtime.h>

#include <cstdint>

#include "rm_device.cuh"

namespace probe {

struct F3 {
  float x, y, z;
};
struct F4 {
  float x, y, z, w;
};
__device__ __forceinline__ F4 sub4(F4 a, F4 b) { return F4{a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
__device__ __forceinline__ float dot4(F4 a, F4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 mul3(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 add3(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }

// glm-shaped vec4 arithmetic (component-wise, then the published reductions)
__device__ __forceinline__ F4 mul4s(F4 a, float s) { return F4{a.x * s, a.y * s, a.z * s, a.w * s}; }
__device__ __forceinline__ F4 add4(F4 a, F4 b) { return F4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
__device__ __forceinline__ F4 mul4(F4 a, F4 b) { return F4{a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
__device__ __forceinline__ F4 matvec(const F4 col[4], F4 v) {
  const F4 m0 = mul4s(col[0], v.x);
  const F4 m1 = mul4s(col[1], v.y);
  const F4 a0 = add4(m0, m1);
  const F4 m2 = mul4s(col[2], v.z);
  const F4 m3 = mul4s(col[3], v.w);
  const F4 a1 = add4(m2, m3);
  return add4(a0, a1);
}
__device__ __forceinline__ float gdot4(F4 a, F4 b) {
  const F4 t = mul4(a, b);
  return (t.x + t.y) + (t.z + t.w);
}
__device__ __forceinline__ F4 gnormalize(F4 v) {
  const float inv = 1.0f / sqrtf(gdot4(v, v));
  return mul4s(v, inv);
}

__global__ void k_d2(const float4* __restrict__ c, const float4* __restrict__ q, int64_t n,
                     float* __restrict__ ref, float* __restrict__ lib) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 a = c[i], b = q[i];
    const F4 diff = sub4(F4{a.x, a.y, a.z, 0.0f}, F4{b.x, b.y, b.z, 0.0f});
    ref[i] = dot4(diff, diff);
    lib[i] = rm::d2_point(a, b.x, b.y, b.z);
  }
}

// o, d: n x 3; t: n
__global__ void k_step(const float* __restrict__ o, const float* __restrict__ d, const float* __restrict__ t,
                       int64_t n, float* __restrict__ ref, float* __restrict__ lib) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const F3 oo{o[3 * i], o[3 * i + 1], o[3 * i + 2]}, dd{d[3 * i], d[3 * i + 1], d[3 * i + 2]};
    const F3 p = add3(oo, mul3(dd, t[i]));
    ref[3 * i] = p.x;
    ref[3 * i + 1] = p.y;
    ref[3 * i + 2] = p.z;
    lib[3 * i] = __fmaf_rn(dd.x, t[i], oo.x);
    lib[3 * i + 1] = __fmaf_rn(dd.y, t[i], oo.y);
    lib[3 * i + 2] = __fmaf_rn(dd.z, t[i], oo.z);
  }
}

// a, b: n x 3
__global__ void k_dot3(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                       float* __restrict__ ref, float* __restrict__ lib) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const F3 x{a[3 * i], a[3 * i + 1], a[3 * i + 2]}, y{b[3 * i], b[3 * i + 1], b[3 * i + 2]};
    ref[i] = dot3(x, y);
    lib[i] = __fmaf_rn(y.z, x.z, __fmaf_rn(x.x, y.x, __fmul_rn(x.y, y.y)));
  }
}

// d2, r: n (step value sqrtf(D) - R)
__global__ void k_stepval(const float* __restrict__ d2, const float* __restrict__ r, int64_t n,
                          float* __restrict__ ref, float* __restrict__ lib) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    ref[i] = sqrtf(d2[i]) - r[i];
    lib[i] = __fsub_rn(__fsqrt_rn(d2[i]), r[i]);
  }
}

// One ray per case: m (n x 16, column-major cam-to-world), wh (n x 2),
// pane (n), xy (n x 2).  Outputs n x 5: dir x, y, z, t_near, t_far.
__global__ void k_ray(const float* __restrict__ m, const int32_t* __restrict__ wh, const float* __restrict__ pane,
                      const int32_t* __restrict__ xy, int64_t n, float* __restrict__ ref, float* __restrict__ lib) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float* mm = m + 16 * i;
    const int W = wh[2 * i], H = wh[2 * i + 1];
    const int x = xy[2 * i], y = xy[2 * i + 1];
    const float P = pane[i];
    // reference form
    const float rx = (float)W, ry = (float)H, cx = (float)x, cy = (float)y;
    const float ux = (2.0f * cx - rx) / 2.0f, uy = (2.0f * cy - ry) / 2.0f;
    const F4 col[4] = {F4{mm[0], mm[1], mm[2], mm[3]}, F4{mm[4], mm[5], mm[6], mm[7]},
                       F4{mm[8], mm[9], mm[10], mm[11]}, F4{mm[12], mm[13], mm[14], mm[15]}};
    const F4 dir4 = gnormalize(matvec(col, F4{ux, uy, -P, 0.0f}));
    const F3 dir{dir4.x, dir4.y, dir4.z};
    // cam_dir = make_float3(-CAMERA_MATRIX[2]): glm's unary minus on a vec4 is
    // vec4(0) -= v, a subtraction from zero per component
    const F3 cam_dir{0.0f - mm[8], 0.0f - mm[9], 0.0f - mm[10]};
    const float dd = dot3(cam_dir, dir);
    float* o = ref + 5 * i;
    o[0] = dir.x;
    o[1] = dir.y;
    o[2] = dir.z;
    o[3] = rm::ZNEAR / dd;
    o[4] = rm::ZFAR / dd;
    // library form
    const rm::Ray r = rm::make_ray(mm, W, H, P, x, y);
    float* l = lib + 5 * i;
    l[0] = r.dx;
    l[1] = r.dy;
    l[2] = r.dz;
    l[3] = r.t_near;
    l[4] = r.t_far;
  }
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

}  // namespace probe

extern "C" {

int fpc_d2(const void* c, const void* q, int64_t n, float* ref, float* lib) {
  probe::k_d2<<<probe::grid_for(n), 256>>>((const float4*)c, (const float4*)q, n, ref, lib);
  return (int)cudaDeviceSynchronize();
}

int fpc_step(const float* o, const float* d, const float* t, int64_t n, float* ref, float* lib) {
  probe::k_step<<<probe::grid_for(n), 256>>>(o, d, t, n, ref, lib);
  return (int)cudaDeviceSynchronize();
}

int fpc_dot3(const float* a, const float* b, int64_t n, float* ref, float* lib) {
  probe::k_dot3<<<probe::grid_for(n), 256>>>(a, b, n, ref, lib);
  return (int)cudaDeviceSynchronize();
}

int fpc_stepval(const float* d2, const float* r, int64_t n, float* ref, float* lib) {
  probe::k_stepval<<<probe::grid_for(n), 256>>>(d2, r, n, ref, lib);
  return (int)cudaDeviceSynchronize();
}

int fpc_ray(const float* m, const int32_t* wh, const float* pane, const int32_t* xy, int64_t n, float* ref,
            float* lib) {
  probe::k_ray<<<probe::grid_for(n), 256>>>(m, wh, pane, xy, n, ref, lib);
  return (int)cudaDeviceSynchronize();
}

}  // extern "C"
