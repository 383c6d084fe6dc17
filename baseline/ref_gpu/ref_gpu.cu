// ref_gpu.cu -- the reference's GPU path restated, as a timed baseline.
//
// Not part of the library: this is what the reference runs on its GPU,
// written again so that it can be built on the GPU host (the reference's own
// FLANN sources cannot travel there) and timed beside the library on the
// same clouds and views.  Nothing here is shared with
// renderer_ray_marching_gb300; the arithmetic is written in the reference's
// source shapes and compiled with nvcc's defaults, as the reference is.
//
// What it restates:
//   - the FLANN CUDA 3-D kd-tree (third_party/flann/algorithms/
//     kdtree_cuda_builder.h:483-599, SplitNodes :270-360,
//     MovePointsToChildNodes :157-226): points kept in x-sorted order (a
//     stable sort by x), every node with more than 64 points (not all equal)
//     split at the midpoint of the longest axis of its tight box, points with
//     a coordinate above the split value going right, stable partitions, so
//     every leaf holds its points in x order; children of a node are
//     neighbours (left, left + 1).  The reference builds it on the GPU with
//     thrust and a host round trip per level; here the same tree is built on
//     the host cores (build time is not part of any figure);
//   - its exact k-NN search (kdtree_cuda_3d_index.cu:52-129, searchNeighbors:
//     stackless descent and backtracking through parent links, far children
//     visited when lastNode == bestChild and their box distance <= the
//     current worst), the result set KnnResultSet<float, useHeap>
//     (util/cuda/result_set.h:121-223) with its heap sort (util/cuda/heap.h),
//     results in global memory;
//   - nearestKernel (kdtree_cuda_3d_index.cu:132-154) for the radii's 2-NN,
//     128 threads per block, plus map_indices (:160-173) and the sqrt of the
//     second distance on the device (the reference's own sqrt is a host loop
//     over device_reference elements, main.cu:110-112, timed separately);
//   - the render kernel (src/ray_marching.cu:63-91) with ray_march (:202-228)
//     and distance_function (:260-292): one thread per pixel in 16 x 16
//     blocks, per step a query written to global memory, a 10-NN search into
//     per-pixel global result arrays, then the min of sqrtf(d2) - r over them
//     (VIND and RADII gathered); the GL surface is replaced by hit-index and
//     depth arrays.  glm 0.9.9.8's mat4 * vec4, dot, normalize and vec4
//     unary minus are written with their published algorithms.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

namespace refgpu {

constexpr float ZFAR = 100.0f;      // src/common.h:4
constexpr float ZNEAR = 0.1f;       // src/common.h:5
constexpr int MAX_STEPS = 128;      // src/common.h:6
constexpr float MIN_DIST = 0.001f;  // src/common.h:7
constexpr int KNN = 10;             // src/ray_marching.h:17
constexpr int LEAF_MAX = 64;        // kdtree_cuda_3d_index.h:55

// kdtree_cuda_builder.h:102-119: a leaf holds its point range, an inner node
// its split axis and value
struct SplitInfo {
  union {
    struct {
      int left;
      int right;
    };
    struct {
      int split_dim;
      float split_val;
    };
  };
};

// ---------------------------------------------------------------- device

// CudaL2 (kdtree_cuda_3d_index.cu:176-193): dot(a - b, a - b) over float4
__device__ __forceinline__ float l2_dist(const float4& a, const float4& b) {
  const float4 d = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
  return d.x * d.x + d.y * d.y + d.z * d.z + d.w * d.w;
}
__device__ __forceinline__ float axis_dist(float a, float b) { return (a - b) * (a - b); }

__device__ __forceinline__ void sift_down(float* key, int* val, int begin, int length) {
  while (2 * begin + 1 < length) {
    const int left = 2 * begin + 1, right = 2 * begin + 2;
    int largest = begin;
    if (left < length && key[left] > key[largest]) largest = left;
    if (right < length && key[right] > key[largest]) largest = right;
    if (largest == begin) return;
    const float tk = key[begin];
    key[begin] = key[largest];
    key[largest] = tk;
    const int tv = val[begin];
    val[begin] = val[largest];
    val[largest] = tv;
    begin = largest;
  }
}

__device__ __forceinline__ void make_heap(float* key, int* val, int length) {
  for (int i = length / 2 - 1; i >= 0; --i) sift_down(key, val, i, length);
}

// KnnResultSet<float, useHeap> with sorted results, in global memory
template <bool UseHeap>
struct ResultSet {
  int found;
  float largest;
  int max_index;
  int k;
  float* dist;
  int* index;

  __device__ void set_location(float* d, int* i, int kk) {
    found = 0;
    largest = INFINITY;
    max_index = 0;
    k = kk;
    dist = d;
    index = i;
    for (int j = 0; j < k; ++j) {
      dist[j] = INFINITY;
      index[j] = -1;
    }
  }
  __device__ float worst() const { return largest; }
  __device__ void find_largest() {
    largest = dist[0];
    max_index = 0;
    for (int j = 1; j < k; ++j)
      if (dist[j] > largest) {
        max_index = j;
        largest = dist[j];
      }
  }
  __device__ void insert(int i, float d) {
    if (found < k) {
      dist[found] = d;
      index[found] = i;
      if (found == k - 1) {
        if (UseHeap) {
          make_heap(dist, index, k);
          largest = dist[0];
        } else {
          find_largest();
        }
      }
      ++found;
    } else if (d < largest) {
      if (UseHeap) {
        dist[0] = d;
        index[0] = i;
        sift_down(dist, index, 0, k);
        largest = dist[0];
      } else {
        dist[max_index] = d;
        index[max_index] = i;
        find_largest();
      }
    }
  }
  __device__ void finish() {
    if (!UseHeap) make_heap(dist, index, k);
    for (int j = k - 1; j > 0; --j) {
      const float td = dist[0];
      dist[0] = dist[j];
      dist[j] = td;
      const int ti = index[0];
      index[0] = index[j];
      index[j] = ti;
      sift_down(dist, index, 0, j);
    }
  }
};

struct TreeDev {
  const SplitInfo* splits;
  const int* child1;
  const int* parent;
  const float4* aabb_min;
  const float4* aabb_max;
  const float4* elements;  // points in tree order, w = 0
  const int* vind;         // tree order -> cloud index
};

template <class RS>
__device__ void search_neighbors(const TreeDev& t, const float4& q, RS& result) {
  bool backtrack = false;
  int last = -1;
  int current = 0;
  while (true) {
    if (current == -1) break;
    const SplitInfo split = t.splits[current];
    float diff = 0.0f;
    if (split.split_dim == 0) diff = q.x - split.split_val;
    else if (split.split_dim == 1) diff = q.y - split.split_val;
    else if (split.split_dim == 2) diff = q.z - split.split_val;
    const int left_child = t.child1[current];
    int best = left_child, other = left_child;
    if (diff < 0) ++other;
    else ++best;
    if (!backtrack) {
      if (left_child == -1) {
        for (int i = split.left; i < split.right; ++i) result.insert(i, l2_dist(t.elements[i], q));
        backtrack = true;
        last = current;
        current = t.parent[current];
      } else {
        last = current;
        current = best;
      }
    } else {
      float mind = 0.0f;
      const float4 lo = t.aabb_min[other], hi = t.aabb_max[other];
      if (q.x < lo.x) mind += axis_dist(q.x, lo.x);
      else if (q.x > hi.x) mind += axis_dist(q.x, hi.x);
      if (q.y < lo.y) mind += axis_dist(q.y, lo.y);
      else if (q.y > hi.y) mind += axis_dist(q.y, hi.y);
      if (q.z < lo.z) mind += axis_dist(q.z, lo.z);
      else if (q.z > hi.z) mind += axis_dist(q.z, hi.z);
      if (last == best && mind <= result.worst()) {
        last = current;
        current = other;
        backtrack = false;
      } else {
        last = current;
        current = t.parent[current];
      }
    }
  }
}

// nearestKernel with KnnResultSet<float, true> (k = 2, sorted), then
// map_indices and the sqrt of the second distance
__global__ void k_radii(TreeDev t, const float4* __restrict__ query, int n, int* __restrict__ res_index,
                        float* __restrict__ res_dist, float* __restrict__ radii, int* __restrict__ nn) {
  const size_t tid = (size_t)blockDim.x * blockIdx.x + threadIdx.x;
  if (tid >= (size_t)n) return;
  const float4 q = make_float4(query[tid].x, query[tid].y, query[tid].z, 0.0f);
  ResultSet<true> rs;
  rs.set_location(res_dist + 2 * tid, res_index + 2 * tid, 2);
  search_neighbors(t, q, rs);
  rs.finish();
  const int j = res_index[2 * tid + 1];
  nn[tid] = j >= 0 ? t.vind[j] : j;
  radii[tid] = sqrtf(res_dist[2 * tid + 1]);
}

// glm 0.9.9.8, published algorithms, vec4 = float4
__device__ __forceinline__ float4 g_add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 g_scale(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ float4 g_mat_vec(const float* m, float4 v) {
  const float4 c0 = make_float4(m[0], m[1], m[2], m[3]), c1 = make_float4(m[4], m[5], m[6], m[7]);
  const float4 c2 = make_float4(m[8], m[9], m[10], m[11]), c3 = make_float4(m[12], m[13], m[14], m[15]);
  const float4 a0 = g_add(g_scale(c0, v.x), g_scale(c1, v.y));
  const float4 a1 = g_add(g_scale(c2, v.z), g_scale(c3, v.w));
  return g_add(a0, a1);
}
__device__ __forceinline__ float g_dot(float4 a, float4 b) {
  const float4 t = make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w);
  return (t.x + t.y) + (t.z + t.w);
}
__device__ __forceinline__ float4 g_normalize(float4 v) { return g_scale(v, 1.0f / sqrtf(g_dot(v, v))); }
__device__ __forceinline__ float4 g_neg(float4 v) {
  return make_float4(0.0f - v.x, 0.0f - v.y, 0.0f - v.z, 0.0f - v.w);  // vec4(0) -= v
}
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct ViewDev {
  float m[16];  // column-major cam-to-world (CAMERA_MATRIX)
  float fov;    // FOV_RADIANS
  int width, height;
};

struct Scratch {
  int* indices;     // W*H*KNN (INDICES)
  float* distances; // W*H*KNN (DISTANCES)
  float4* query;    // W*H (QUERY)
};

struct Hit {
  float distance;
  int index;
};

// distance_function, src/ray_marching.cu:260-292
__device__ Hit distance_function(const TreeDev& t, const float* radii, const Scratch& s, float3 pos, int lin) {
  Hit hit{1.0f / 0.0f, 0};
  const int off = lin * KNN;
  s.query[lin] = make_float4(pos.x, pos.y, pos.z, 0.0f);
  ResultSet<false> rs;
  rs.set_location(s.distances + off, s.indices + off, KNN);
  search_neighbors(t, s.query[lin], rs);
  rs.finish();
  for (int i = 0; i < KNN; ++i) {
    const int ii = s.indices[off + i];
    const int index = ii >= 0 ? t.vind[ii] : ii;
    if (index < 0) continue;
    const float dist = sqrtf(s.distances[off + i]) - radii[index];
    if (dist < hit.distance) {  // is_inside() returns true (its body is commented out)
      hit.distance = dist;
      hit.index = index;
    }
  }
  return hit;
}

// render + ray_march, src/ray_marching.cu:63-91, 202-228
__global__ void k_render(TreeDev t, const float* __restrict__ radii, ViewDev v, Scratch s, int* __restrict__ hit_out,
                         float* __restrict__ depth_out) {
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= v.width || y >= v.height) return;
  const float rx = (float)v.width, ry = (float)v.height, cx = (float)x, cy = (float)y;
  const float ux = (2.0f * cx - rx) / 2.0f, uy = (2.0f * cy - ry) / 2.0f;
  const float pane = (float)v.width / (2.0f * tanf(0.5f * v.fov));
  const float4 cam_dir4 = g_neg(make_float4(v.m[8], v.m[9], v.m[10], v.m[11]));
  const float3 cam_dir = make_float3(cam_dir4.x, cam_dir4.y, cam_dir4.z);
  const float3 origin = make_float3(v.m[12], v.m[13], v.m[14]);
  const float4 d4 = g_normalize(g_mat_vec(v.m, make_float4(ux, uy, -pane, 0.0f)));
  const float3 dir = make_float3(d4.x, d4.y, d4.z);
  const float far_d = ZFAR / dot3(cam_dir, dir);
  const float near_d = ZNEAR / dot3(cam_dir, dir);
  const int lin = y * v.width + x;
  float t_total = near_d;
  int index = -1;
  float depth = 0.0f;
  for (int i = 0; i < MAX_STEPS; ++i) {
    const float3 p = make_float3(origin.x + dir.x * t_total, origin.y + dir.y * t_total, origin.z + dir.z * t_total);
    const Hit h = distance_function(t, radii, s, p, lin);
    t_total += h.distance;
    if (h.distance < MIN_DIST) {
      depth = t_total;
      index = h.index;
      break;
    }
    if (t_total > far_d) break;
  }
  hit_out[lin] = index;
  depth_out[lin] = index >= 0 ? depth : 0.0f;
}

// ------------------------------------------------------------------ host

struct Tree {
  std::vector<SplitInfo> splits;
  std::vector<int> child1, parent;
  std::vector<float4> amin, amax;
  std::vector<float4> elements;
  std::vector<int> vind;
};

static void node_box(const float* xyz, const int* ids, int lo, int hi, float4& mn, float4& mx) {
  mn = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
  mx = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
  for (int i = lo; i < hi; ++i) {
    const float* p = xyz + 3 * (size_t)ids[i];
    mn.x = std::min(mn.x, p[0]);
    mn.y = std::min(mn.y, p[1]);
    mn.z = std::min(mn.z, p[2]);
    mx.x = std::max(mx.x, p[0]);
    mx.y = std::max(mx.y, p[1]);
    mx.z = std::max(mx.z, p[2]);
  }
}

// The FLANN CUDA kd-tree over n points (xyz, stride 3), built level by level
// as CudaKdTreeBuilder::buildTree does.
static void build_tree(const float* xyz, int n, Tree& t) {
  std::vector<int> ids(n);
  std::iota(ids.begin(), ids.end(), 0);
  std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return xyz[3 * (size_t)a] < xyz[3 * (size_t)b]; });
  t.splits.assign(1, SplitInfo{});
  t.child1.assign(1, -1);
  t.parent.assign(1, -1);
  t.amin.resize(1);
  t.amax.resize(1);
  t.splits[0].left = 0;
  t.splits[0].right = n;
  node_box(xyz, ids.data(), 0, n, t.amin[0], t.amax[0]);
  std::vector<int> level{0}, next;
  std::vector<int> tmp;
  while (!level.empty()) {
    next.clear();
    for (int node : level) {
      const int lo = t.splits[node].left, hi = t.splits[node].right;
      const float4 mn = t.amin[node], mx = t.amax[node];
      const bool all_equal = mn.x == mx.x && mn.y == mx.y && mn.z == mx.z;
      if (hi - lo <= LEAF_MAX || all_equal) continue;
      // SplitNodes: the midpoint of the longest extent (the first on ties)
      const float ext[3] = {mx.x - mn.x, mx.y - mn.y, mx.z - mn.z};
      const float mid[3] = {(mx.x + mn.x) * 0.5f, (mx.y + mn.y) * 0.5f, (mx.z + mn.z) * 0.5f};
      int dim = 0;
      float len = ext[0];
      for (int a = 1; a <= 2; ++a)
        if (ext[a] > len) {
          dim = a;
          len = ext[a];
        }
      const float val = mid[dim];
      // MovePointsToChildNodes + separate_left_and_right_children: a stable
      // partition, coordinate > split value to the right
      tmp.clear();
      int nl = 0;
      for (int i = lo; i < hi; ++i)
        if (!(xyz[3 * (size_t)ids[i] + dim] > val)) ids[lo + nl++] = ids[i];
        else tmp.push_back(ids[i]);
      std::copy(tmp.begin(), tmp.end(), ids.begin() + lo + nl);
      const int left = (int)t.splits.size();
      t.splits.resize(left + 2);
      t.child1.resize(left + 2, -1);
      t.parent.resize(left + 2, node);
      t.amin.resize(left + 2);
      t.amax.resize(left + 2);
      t.child1[node] = left;
      t.splits[node].split_dim = dim;
      t.splits[node].split_val = val;
      t.splits[left].left = lo;
      t.splits[left].right = lo + nl;
      t.splits[left + 1].left = lo + nl;
      t.splits[left + 1].right = hi;
      node_box(xyz, ids.data(), lo, lo + nl, t.amin[left], t.amax[left]);
      node_box(xyz, ids.data(), lo + nl, hi, t.amin[left + 1], t.amax[left + 1]);
      next.push_back(left);
      next.push_back(left + 1);
    }
    level.swap(next);
  }
  t.elements.resize(n);
  t.vind = ids;
  for (int i = 0; i < n; ++i) {
    const float* p = xyz + 3 * (size_t)ids[i];
    t.elements[i] = make_float4(p[0], p[1], p[2], 0.0f);
  }
}

template <class T>
static T* upload(const std::vector<T>& v, cudaError_t& e) {
  T* p = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&p, std::max<size_t>(1, v.size()) * sizeof(T));
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return p;
}

struct Handle {
  int n = 0;
  int nodes = 0;
  TreeDev t{};
  void* bufs[7] = {};
  float4* query = nullptr;  // the points themselves (main.cu:91-92)
  float* radii = nullptr;   // clamped render radii, cloud order
  Scratch s{};
  size_t scratch_pixels = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::string err;
};

}  // namespace refgpu

using namespace refgpu;

extern "C" {

// Builds the tree over n points (xyz, host memory) and uploads it.
void* rg_create(const float* xyz, int n) {
  Handle* h = new Handle();
  h->n = n;
  Tree t;
  build_tree(xyz, n, t);
  h->nodes = (int)t.splits.size();
  cudaError_t e = cudaSuccess;
  SplitInfo* sp = upload(t.splits, e);
  int* c1 = upload(t.child1, e);
  int* pa = upload(t.parent, e);
  float4* mn = upload(t.amin, e);
  float4* mx = upload(t.amax, e);
  float4* el = upload(t.elements, e);
  int* vi = upload(t.vind, e);
  std::vector<float4> q(n);
  for (int i = 0; i < n; ++i) q[i] = make_float4(xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2], 0.0f);
  h->query = upload(q, e);
  if (e == cudaSuccess) e = cudaMalloc(&h->radii, std::max(1, n) * sizeof(float));
  if (e == cudaSuccess) e = cudaEventCreate(&h->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&h->e1);
  h->t = TreeDev{sp, c1, pa, mn, mx, el, vi};
  void* b[7] = {sp, c1, pa, mn, mx, el, vi};
  memcpy(h->bufs, b, sizeof(b));
  if (e != cudaSuccess) h->err = cudaGetErrorString(e);
  return h;
}

const char* rg_error(void* hp) { return static_cast<Handle*>(hp)->err.c_str(); }
int rg_nodes(void* hp) { return static_cast<Handle*>(hp)->nodes; }

// The radii precompute on the device (nearestKernel k = 2 over the points,
// map_indices, sqrt); radii_out / nn_out are host arrays of n.  Returns the
// kernel time in ms (CUDA events), or a negative value on error.
float rg_radii(void* hp, float max_radius, float* radii_out, int* nn_out) {
  Handle* h = static_cast<Handle*>(hp);
  int* ri = nullptr;
  float* rd = nullptr;
  float* rr = nullptr;
  int* nn = nullptr;
  cudaError_t e = cudaMalloc(&ri, 2 * (size_t)h->n * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&rd, 2 * (size_t)h->n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&rr, (size_t)h->n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&nn, (size_t)h->n * sizeof(int));
  float ms = -1.0f;
  if (e == cudaSuccess) {
    const int threads = 128;
    const int blocks = (h->n + threads - 1) / threads;
    cudaEventRecord(h->e0);
    k_radii<<<blocks, threads>>>(h->t, h->query, h->n, ri, rd, rr, nn);
    cudaEventRecord(h->e1);
    e = cudaEventSynchronize(h->e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, h->e0, h->e1);
  }
  if (e == cudaSuccess && radii_out) e = cudaMemcpy(radii_out, rr, (size_t)h->n * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nn_out) e = cudaMemcpy(nn_out, nn, (size_t)h->n * 4, cudaMemcpyDeviceToHost);
  // render radii: min(r, max_radius) in cloud order (main.cu:144-149); the
  // kernel wrote them in cloud order already (the queries are the cloud)
  if (e == cudaSuccess) {
    std::vector<float> r((size_t)h->n);
    e = cudaMemcpy(r.data(), rr, (size_t)h->n * 4, cudaMemcpyDeviceToHost);
    for (auto& x : r)
      if (max_radius > 0.0f && x > max_radius) x = max_radius;
    if (e == cudaSuccess) e = cudaMemcpy(h->radii, r.data(), (size_t)h->n * 4, cudaMemcpyHostToDevice);
  }
  cudaFree(ri);
  cudaFree(rd);
  cudaFree(rr);
  cudaFree(nn);
  if (e != cudaSuccess) {
    h->err = cudaGetErrorString(e);
    return -1.0f;
  }
  return ms;
}

// The reference's radii post-process as shipped (main.cu:110-112): a host
// loop over thrust device_reference elements, one synchronous 4-byte copy
// from the device and one back per point.  Runs it over the first `count`
// points of a scratch copy and returns the seconds it took (the caller
// scales this per point; at 10^7 points the loop takes minutes).
double rg_sqrt_loop_sample(void* hp, int count) {
  Handle* h = static_cast<Handle*>(hp);
  count = std::min(count, h->n);
  float* d = nullptr;
  if (cudaMalloc(&d, 2 * (size_t)std::max(count, 1) * sizeof(float)) != cudaSuccess) return -1.0;
  cudaMemset(d, 0, 2 * (size_t)std::max(count, 1) * sizeof(float));
  cudaDeviceSynchronize();
  const auto t0 = std::chrono::steady_clock::now();
  for (int i = 1; i < 2 * count; i += 2) {
    float v;
    cudaMemcpy(&v, d + i, sizeof(float), cudaMemcpyDeviceToHost);
    v = std::sqrt(v);
    cudaMemcpy(d + i / 2, &v, sizeof(float), cudaMemcpyHostToDevice);
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  cudaFree(d);
  return secs;
}

// Render radii given in cloud order (host array of n), already clamped.
int rg_set_radii(void* hp, const float* radii) {
  Handle* h = static_cast<Handle*>(hp);
  const cudaError_t e = cudaMemcpy(h->radii, radii, (size_t)h->n * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) h->err = cudaGetErrorString(e);
  return (int)e;
}

// One view (render_to_texture): cam2world column-major, width, height, fov;
// hit_out / depth_out are DEVICE arrays of width*height.  Returns the kernel
// time in ms, or a negative value on error.
float rg_render(void* hp, const float* cam2world, int width, int height, float fov, int* hit_out,
                float* depth_out) {
  Handle* h = static_cast<Handle*>(hp);
  const size_t pix = (size_t)width * height;
  cudaError_t e = cudaSuccess;
  if (pix > h->scratch_pixels) {  // render_to_texture resizes its scratch (ray_marching.cu:98-103)
    cudaFree(h->s.indices);
    cudaFree(h->s.distances);
    cudaFree(h->s.query);
    h->s = Scratch{};
    e = cudaMalloc(&h->s.indices, pix * KNN * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h->s.distances, pix * KNN * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&h->s.query, pix * sizeof(float4));
    h->scratch_pixels = e == cudaSuccess ? pix : 0;
  }
  float ms = -1.0f;
  if (e == cudaSuccess) {
    ViewDev v;
    memcpy(v.m, cam2world, sizeof(v.m));
    v.fov = fov;
    v.width = width;
    v.height = height;
    dim3 block(16, 16, 1);
    dim3 grid((width + 15) / 16, (height + 15) / 16, 1);
    cudaEventRecord(h->e0);
    k_render<<<grid, block>>>(h->t, h->radii, v, h->s, hit_out, depth_out);
    cudaEventRecord(h->e1);
    e = cudaEventSynchronize(h->e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, h->e0, h->e1);
  }
  if (e != cudaSuccess) {
    h->err = cudaGetErrorString(e);
    return -1.0f;
  }
  return ms;
}

void rg_destroy(void* hp) {
  Handle* h = static_cast<Handle*>(hp);
  if (!h) return;
  for (void* p : h->bufs) cudaFree(p);
  cudaFree(h->query);
  cudaFree(h->radii);
  cudaFree(h->s.indices);
  cudaFree(h->s.distances);
  cudaFree(h->s.query);
  if (h->e0) cudaEventDestroy(h->e0);
  if (h->e1) cudaEventDestroy(h->e1);
  delete h;
}

}  // extern "C"
