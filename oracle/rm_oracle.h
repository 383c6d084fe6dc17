/*
 * rm_oracle.h -- CPU oracle for the renderer hot path (TEST INFRASTRUCTURE).
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check in __graft_entry__.py and the CPU-baseline leg of bench.py load it.
 * It restates, in plain C with every rounding step written out, what the
 * reference computes on its GPU path:
 *
 *   - radii: 2-NN including self over the cloud, radius = sqrtf(d2 of the
 *     second entry), clamped to max_radius when max_radius > 0
 *     (reference main.cu:102-113 and main.cu:144-149);
 *   - the marcher: pinhole ray generation (src/ray_marching.cu:63-81),
 *     sphere tracing with MAX_STEPS=128 / MIN_DIST=1e-3 / near-far planes
 *     (src/ray_marching.cu:202-228, src/common.h:4-11), and the distance
 *     function "min over the 10 nearest centres of sqrtf(d2) - radius"
 *     (src/ray_marching.cu:260-292, k=10 from src/ray_marching.h:17);
 *   - the first-hit depth surrogate used for gradients (no reference
 *     counterpart; the reference has no backward pass).
 *
 * Floating point contract (identical in the CUDA kernels):
 *   d2(c, q)  = fmaf(dz, dz, fmaf(dx, dx, dy*dy)), d = c - q   (FLANN CudaL2::dist,
 *               kdtree_cuda_3d_index.cu:186-192, as nvcc contracts it)
 *   p(t)      = fmaf(dir, t, o) per component       (ray_marching.cu:216)
 *   dot3(a,b) = fmaf(az, bz, fmaf(ax, bx, ay*by))   (ray_marching.cu:78-79)
 *   mat*vec   = fmaf(c0, x, c1*y) + fmaf(c2, z, c3*w) per row (glm column sum)
 *   |v|^2     = fmaf(x, x, y*y) + fmaf(z, z, w*w), normalize = v * (1/sqrtf(|v|^2))
 * The library is compiled with -ffp-contract=off so the C compiler adds no
 * contraction of its own on either x86-64 or aarch64.
 *
 * Nearest-neighbour order is (d2, original index) ascending: equal squared
 * distances are broken by the lower point index.
 */
#ifndef RM_ORACLE_H
#define RM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rmo_index rmo_index;

typedef struct {
  float cam2world[16]; /* column-major 4x4 (column c at [4c..4c+3]) */
  int32_t width;
  int32_t height;
  float pane;          /* W / (2 tan(fov/2)), resolved per view */
} rmo_view;

/* Build an exact kNN index over n points given as xyz triplets (stride 3). */
rmo_index* rmo_index_build(const float* xyz, int64_t n);
void rmo_index_free(rmo_index* ix);

/* k nearest neighbours (k <= 32) of m query points; rows padded with
 * idx=-1, d2=+inf when the cloud has fewer than k points. */
void rmo_knn(const rmo_index* ix, const float* q, int64_t m, int k,
             int32_t* idx_out, float* d2_out, int threads);

/* Radii: sqrtf of the second entry of each point's self-inclusive 2-NN list,
 * clamped to max_radius when max_radius > 0.  nn_out gets that entry's
 * index (-1 when n == 1). */
void rmo_radii(const rmo_index* ix, float max_radius, float* radii_out,
               int32_t* nn_out, int threads);

/* March the given pixels (linear index y*W + x, y = 0 is the bottom row) of
 * one view.  radii are per point in original order.  Outputs per listed
 * pixel: hit index (-1 for background), depth (0 for background), step
 * count (number of distance-function evaluations). */
void rmo_render(const rmo_index* ix, const float* radii, const rmo_view* v,
                const int64_t* pixels, int64_t npix, int32_t* hit_out,
                float* depth_out, int32_t* steps_out, int threads);

/* One distance-function evaluation at p (xyz): returns the step value and
 * writes the chosen index (0 when no candidate exists, as the reference's
 * default RayHit). */
float rmo_distance(const rmo_index* ix, const float* radii, const float* p,
                   int32_t* idx_out);

/* Ray of pixel (x, y): origin, unit direction, near and far distances. */
void rmo_ray(const rmo_view* v, int32_t x, int32_t y, float* o, float* d,
             float* t_near, float* t_far);

/* Analytic entry distance of ray (o, d) into sphere (c, r) in double
 * precision, with the gradient w.r.t. c (3) and r (1).  Returns the
 * discriminant (negative: the ray misses the sphere; the depth is then the
 * closest-approach distance and the gradients are d and 0). */
double rmo_sphere_depth(const double* o, const double* d, const double* c,
                        double r, double* t_out, double* g_c, double* g_r);

#ifdef __cplusplus
}
#endif
#endif
