/*
 * rm_oracle.c -- CPU oracle for the renderer hot path (TEST INFRASTRUCTURE,
 * never linked into the product).  See rm_oracle.h for the floating-point
 * contract and the reference lines each function restates.
 *
 * The exact kNN uses a plain median-split kd-tree written for this oracle
 * (not FLANN's): the answer is the mathematically defined (d2, index)-ordered
 * k-set, so the tree shape does not matter.  Pruning compares a lower bound
 * computed with the same monotone d2 formula, visiting a subtree whenever
 * its bound is <= the current k-th distance, so ties are never lost.
 *
 * Build with -O2 -ffp-contract=off (-fopenmp optional).
 */
#include "rm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RMO_LEAF 8
#define RMO_MAXK 32
#define RMO_ZFAR 100.0f      /* src/common.h:4 */
#define RMO_ZNEAR 0.1f       /* src/common.h:5 */
#define RMO_MAX_STEPS 128    /* src/common.h:6 */
#define RMO_MIN_DIST 0.001f  /* src/common.h:7 */
#define RMO_KNN 10           /* src/ray_marching.h:17 */

typedef struct {
  float lo[3], hi[3];
  int32_t left;   /* child index, or -1 for a leaf */
  int32_t right;
  int64_t start;  /* leaf: range in ix->order */
  int64_t count;
} rmo_node;

struct rmo_index {
  int64_t n;
  float* xyz;      /* copy of the points, stride 3 */
  int64_t* order;  /* point ids grouped by leaf */
  rmo_node* nodes;
  int64_t nnodes;
};

/* Squared distance, FLANN CudaL2::dist order as nvcc contracts it. */
static inline float d2f(float cx, float cy, float cz, float qx, float qy,
                        float qz) {
  float dx = cx - qx, dy = cy - qy, dz = cz - qz;
  return fmaf(dz, dz, fmaf(dx, dx, dy * dy));
}

/* Lower bound of d2f over a box: per-axis gaps are monotone in |c - q|. */
static inline float box_d2(const rmo_node* nd, const float* q) {
  float g[3];
  for (int a = 0; a < 3; ++a) {
    if (q[a] < nd->lo[a]) g[a] = nd->lo[a] - q[a];
    else if (q[a] > nd->hi[a]) g[a] = q[a] - nd->hi[a];
    else g[a] = 0.0f;
  }
  return fmaf(g[2], g[2], fmaf(g[0], g[0], g[1] * g[1]));
}

/* Nodes of a subtree over `count` points: the split is always count/2, so
 * the tree shape (and a pre-order numbering) depends on the count alone,
 * which lets independent subtrees be built in parallel. */
static void nodes_pair(int64_t m, int64_t* a, int64_t* b) {
  /* a = nodes(m), b = nodes(m + 1), with nodes(c) = 1 for c <= LEAF,
   * nodes(2k) = 1 + 2 nodes(k), nodes(2k + 1) = 1 + nodes(k) + nodes(k + 1) */
  if (m + 1 <= RMO_LEAF) { *a = 1; *b = 1; return; }
  int64_t k = m / 2, nk, nk1;
  nodes_pair(k, &nk, &nk1);
  if (m % 2 == 0) {
    *a = (m <= RMO_LEAF) ? 1 : 1 + 2 * nk;
    *b = 1 + nk + nk1;
  } else {
    *a = (m <= RMO_LEAF) ? 1 : 1 + nk + nk1;
    *b = 1 + 2 * nk1;
  }
}

static int64_t subtree_nodes(int64_t count) {
  int64_t a, b;
  nodes_pair(count, &a, &b);
  return a;
}

/* Quickselect on order[lo, hi) by coordinate `axis`, k-th element in place. */
static void select_axis(const float* xyz, int64_t* order, int64_t lo, int64_t hi,
                        int64_t k, int axis) {
  while (hi - lo > 1) {
    int64_t mid = lo + (hi - lo) / 2;
    float pv = xyz[order[mid] * 3 + axis];
    int64_t i = lo, j = hi - 1;
    while (i <= j) {
      while (xyz[order[i] * 3 + axis] < pv) ++i;
      while (xyz[order[j] * 3 + axis] > pv) --j;
      if (i <= j) {
        int64_t t = order[i]; order[i] = order[j]; order[j] = t;
        ++i; --j;
      }
    }
    if (k <= j) hi = j + 1;
    else if (k >= i) lo = i;
    else return;
  }
}

static void build_rec(rmo_index* ix, int64_t id, int64_t start, int64_t count) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = start; i < start + count; ++i) {
    const float* p = ix->xyz + ix->order[i] * 3;
    for (int a = 0; a < 3; ++a) {
      if (p[a] < lo[a]) lo[a] = p[a];
      if (p[a] > hi[a]) hi[a] = p[a];
    }
  }
  rmo_node* nd = &ix->nodes[id];
  memcpy(nd->lo, lo, sizeof lo);
  memcpy(nd->hi, hi, sizeof hi);
  nd->start = start;
  nd->count = count;
  nd->left = nd->right = -1;
  if (count <= RMO_LEAF) return;
  int axis = 0;
  float ext = hi[0] - lo[0];
  for (int a = 1; a < 3; ++a)
    if (hi[a] - lo[a] > ext) { ext = hi[a] - lo[a]; axis = a; }
  int64_t half = count / 2;
  select_axis(ix->xyz, ix->order, start, start + count, start + half, axis);
  int64_t l = id + 1;
  int64_t r = id + 1 + subtree_nodes(half);
  nd->left = (int32_t)l;
  nd->right = (int32_t)r;
  if (count > (1 << 16)) {
#pragma omp task default(shared) firstprivate(l, start, half)
    build_rec(ix, l, start, half);
#pragma omp task default(shared) firstprivate(r, start, half, count)
    build_rec(ix, r, start + half, count - half);
#pragma omp taskwait
  } else {
    build_rec(ix, l, start, half);
    build_rec(ix, r, start + half, count - half);
  }
}

rmo_index* rmo_index_build(const float* xyz, int64_t n) {
  rmo_index* ix = (rmo_index*)calloc(1, sizeof(rmo_index));
  ix->n = n;
  ix->xyz = (float*)malloc((size_t)(n > 0 ? n : 1) * 3 * sizeof(float));
  ix->order = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  if (n > 0) memcpy(ix->xyz, xyz, (size_t)n * 3 * sizeof(float));
  for (int64_t i = 0; i < n; ++i) ix->order[i] = i;
  if (n > 0) {
    ix->nnodes = subtree_nodes(n);
    ix->nodes = (rmo_node*)malloc((size_t)ix->nnodes * sizeof(rmo_node));
#pragma omp parallel
#pragma omp single
    build_rec(ix, 0, 0, n);
  }
  return ix;
}

void rmo_index_free(rmo_index* ix) {
  if (!ix) return;
  free(ix->xyz);
  free(ix->order);
  free(ix->nodes);
  free(ix);
}

/* (d2, index) strictly-less */
static inline int knn_less(float da, int64_t ia, float db, int64_t ib) {
  return da < db || (da == db && ia < ib);
}

/* Exact k-NN of q; writes k sorted entries (padding -1 / +inf). */
static void knn_query(const rmo_index* ix, const float* q, int k, int32_t* oi,
                      float* od) {
  float bd[RMO_MAXK];
  int64_t bi[RMO_MAXK];
  int cnt = 0;
  for (int j = 0; j < k; ++j) { bd[j] = INFINITY; bi[j] = -1; }
  if (ix->n > 0) {
    int32_t stack[128];
    float sd[128];
    int sp = 0;
    stack[sp] = 0; sd[sp] = 0.0f; ++sp;
    while (sp > 0) {
      --sp;
      int32_t nid = stack[sp];
      float md = sd[sp];
      float worst = cnt < k ? INFINITY : bd[k - 1];
      if (md > worst) continue;
      const rmo_node* nd = &ix->nodes[nid];
      if (nd->left < 0) {
        for (int64_t i = nd->start; i < nd->start + nd->count; ++i) {
          int64_t pid = ix->order[i];
          const float* c = ix->xyz + pid * 3;
          float d = d2f(c[0], c[1], c[2], q[0], q[1], q[2]);
          if (cnt < k || knn_less(d, pid, bd[k - 1], bi[k - 1])) {
            int j = cnt < k ? cnt : k - 1;
            while (j > 0 && knn_less(d, pid, bd[j - 1], bi[j - 1])) {
              bd[j] = bd[j - 1]; bi[j] = bi[j - 1]; --j;
            }
            bd[j] = d; bi[j] = pid;
            if (cnt < k) ++cnt;
          }
        }
      } else {
        const rmo_node* a = &ix->nodes[nd->left];
        const rmo_node* b = &ix->nodes[nd->right];
        float da = box_d2(a, q), db = box_d2(b, q);
        /* push the farther child first so the nearer one is expanded next */
        if (da <= db) {
          stack[sp] = nd->right; sd[sp] = db; ++sp;
          stack[sp] = nd->left; sd[sp] = da; ++sp;
        } else {
          stack[sp] = nd->left; sd[sp] = da; ++sp;
          stack[sp] = nd->right; sd[sp] = db; ++sp;
        }
      }
    }
  }
  for (int j = 0; j < k; ++j) { oi[j] = (int32_t)bi[j]; od[j] = bd[j]; }
}

static int nthreads(int threads) {
#ifdef _OPENMP
  return threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

void rmo_knn(const rmo_index* ix, const float* q, int64_t m, int k,
             int32_t* idx_out, float* d2_out, int threads) {
  if (k > RMO_MAXK) k = RMO_MAXK;
  int nt = nthreads(threads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
  for (int64_t i = 0; i < m; ++i)
    knn_query(ix, q + i * 3, k, idx_out + i * k, d2_out + i * k);
}

void rmo_radii(const rmo_index* ix, float max_radius, float* radii_out,
               int32_t* nn_out, int threads) {
  int nt = nthreads(threads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
  for (int64_t i = 0; i < ix->n; ++i) {
    int32_t id[2];
    float d[2];
    knn_query(ix, ix->xyz + i * 3, 2, id, d);
    float r = sqrtf(d[1]);                       /* main.cu:111 */
    if (max_radius > 0.0f && r > max_radius) r = max_radius; /* main.cu:144-149 */
    radii_out[i] = r;
    if (nn_out) nn_out[i] = id[1];
  }
}

/* src/ray_marching.cu:260-292: min over the 10 nearest of sqrtf(d2) - r,
 * visiting candidates in ascending (d2, index) order with a strict "<".
 * The initial best is {+inf, index 0} (RayHit defaults, :43-46). */
static float distance_fn(const rmo_index* ix, const float* radii, const float* p,
                         int32_t* idx) {
  int32_t id[RMO_KNN];
  float d[RMO_KNN];
  knn_query(ix, p, RMO_KNN, id, d);
  float best = INFINITY;
  int32_t bi = 0;
  for (int j = 0; j < RMO_KNN; ++j) {
    if (id[j] < 0) continue;
    float v = sqrtf(d[j]) - radii[id[j]];
    if (v < best) { best = v; bi = id[j]; }
  }
  *idx = bi;
  return best;
}

float rmo_distance(const rmo_index* ix, const float* radii, const float* p,
                   int32_t* idx_out) {
  return distance_fn(ix, radii, p, idx_out);
}

/* src/ray_marching.cu:70-79 with the glm column combination and normalize. */
void rmo_ray(const rmo_view* v, int32_t x, int32_t y, float* o, float* d,
             float* t_near, float* t_far) {
  const float* m = v->cam2world;
  float ux = (2.0f * (float)x - (float)v->width) / 2.0f;
  float uy = (2.0f * (float)y - (float)v->height) / 2.0f;
  float uz = -v->pane;
  float zero = 0.0f;
  float r[4];
  for (int i = 0; i < 4; ++i) {
    float a = fmaf(m[0 + i], ux, m[4 + i] * uy);
    float b = fmaf(m[8 + i], uz, m[12 + i] * zero);
    r[i] = a + b;
  }
  float len2 = fmaf(r[0], r[0], r[1] * r[1]) + fmaf(r[2], r[2], r[3] * r[3]);
  float inv = 1.0f / sqrtf(len2);
  d[0] = r[0] * inv;
  d[1] = r[1] * inv;
  d[2] = r[2] * inv;
  float cd[3] = {-m[8], -m[9], -m[10]};
  float dd = fmaf(cd[2], d[2], fmaf(cd[0], d[0], cd[1] * d[1]));
  *t_far = RMO_ZFAR / dd;
  *t_near = RMO_ZNEAR / dd;
  o[0] = m[12];
  o[1] = m[13];
  o[2] = m[14];
}

void rmo_render(const rmo_index* ix, const float* radii, const rmo_view* v,
                const int64_t* pixels, int64_t npix, int32_t* hit_out,
                float* depth_out, int32_t* steps_out, int threads) {
  int nt = nthreads(threads);
  (void)nt;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
  for (int64_t k = 0; k < npix; ++k) {
    int64_t pix = pixels[k];
    int32_t x = (int32_t)(pix % v->width), y = (int32_t)(pix / v->width);
    float o[3], d[3], tn, tf;
    rmo_ray(v, x, y, o, d, &tn, &tf);
    /* src/ray_marching.cu:202-228 */
    float t = tn;
    int32_t hit = -1, steps = 0;
    float depth = 0.0f;
    for (int i = 0; i < RMO_MAX_STEPS; ++i) {
      float p[3] = {fmaf(d[0], t, o[0]), fmaf(d[1], t, o[1]), fmaf(d[2], t, o[2])};
      int32_t idx;
      float s = distance_fn(ix, radii, p, &idx);
      ++steps;
      t = t + s;
      if (s < RMO_MIN_DIST) { hit = idx; depth = t; break; }
      if (t > tf) break;
    }
    hit_out[k] = hit;
    if (depth_out) depth_out[k] = depth;
    if (steps_out) steps_out[k] = steps;
  }
}

double rmo_sphere_depth(const double* o, const double* d, const double* c,
                        double r, double* t_out, double* g_c, double* g_r) {
  double oc[3] = {c[0] - o[0], c[1] - o[1], c[2] - o[2]};
  double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  double b = d[0] * oc[0] + d[1] * oc[1] + d[2] * oc[2];
  double cc = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - r * r;
  double disc = b * b - a * cc;
  if (disc <= 0.0) {
    *t_out = b / a;
    for (int i = 0; i < 3; ++i) g_c[i] = d[i] / a;
    *g_r = 0.0;
    return disc;
  }
  double s = sqrt(disc);
  *t_out = (b - s) / a;
  for (int i = 0; i < 3; ++i) g_c[i] = (d[i] - (b * d[i] - a * oc[i]) / s) / a;
  *g_r = -r / s;
  return disc;
}
