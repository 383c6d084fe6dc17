// rm_device.cuh -- device-side building blocks shared by the index, radii,
// marcher and backward kernels.
//
// Floating-point contract.  Every operation whose rounding decides a result
// bit is written with an explicit round-to-nearest intrinsic so that the
// compiler cannot contract differently from the reference's GPU build:
//   d2(c, q) = fma(dz, dz, fma(dx, dx, dy*dy)), d = c - q
//       FLANN CudaL2::dist (third_party/flann/algorithms/kdtree_cuda_3d_index.cu:186-192,
//       dot(float4) of util/cutil_math.h:1127-1130 with w = 0) as nvcc contracts it;
//   p(t) = fma(dir, t, o)                    src/ray_marching.cu:216
//   dot3(a, b) = fma(az, bz, fma(ax, bx, ay*by))      src/ray_marching.cu:78-79
//   mat*vec row = fma(c0, x, c1*y) + fma(c2, z, c3*w) glm column sum, :77
//   |v|^2 = fma(x, x, y*y) + fma(z, z, w*w); normalize = v * (1 / sqrt(|v|^2))
// The same expressions are in the CPU oracle, compiled without contraction.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rm {

constexpr int KNN = 10;             // src/ray_marching.h:17
constexpr float ZFAR = 100.0f;      // src/common.h:4
constexpr float ZNEAR = 0.1f;       // src/common.h:5
constexpr int MAX_STEPS = 128;      // src/common.h:6
constexpr float MIN_DIST = 0.001f;  // src/common.h:7
constexpr int MAX_LEVELS = 14;      // 4^14 leaf slots (group offsets stay 32-bit)
constexpr int STACK = 3 * MAX_LEVELS + 4;
constexpr int GROUP_F4 = 8;         // float4 per child group (6 used)

// Index view passed by value to kernels.
struct IndexDev {
  const float4* rec;     // sorted records (x, y, z, radius)
  const float4* col;     // sorted colours (r, g, b, 1)
  const float4* groups;  // child groups: per internal node, its 4 children's boxes
  const int32_t* perm;   // sorted position -> cloud index
  int64_t n;             // points
  int32_t leaf;          // points per leaf
  int32_t depth;         // level of the leaves (>= 1); the root is level 0
};

// Offset of the first child group of level `lvl` (levels 0..depth-1 own
// groups).  32-bit arithmetic: (4^lvl - 1) / 3 fits for lvl <= MAX_LEVELS,
// and a 32-bit division by a constant is a multiply-high where the 64-bit
// one is a multi-instruction sequence on the walk's per-node path.
__host__ __device__ __forceinline__ int64_t group_offset(int lvl) {
  return (int64_t)(((1u << (2 * lvl)) - 1u) / 3u);
}

__device__ __forceinline__ float d2_point(float4 c, float qx, float qy, float qz) {
  float dx = __fsub_rn(c.x, qx);
  float dy = __fsub_rn(c.y, qy);
  float dz = __fsub_rn(c.z, qz);
  return __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
}

// Lower bound of d2_point over a box: each axis gap is fl(|c - q|) of the
// nearest face, which never exceeds fl(|c - q|) for a contained c because
// rounding is monotone; the same fma chain keeps the bound monotone.
__device__ __forceinline__ float d2_box(float lx, float ly, float lz, float hx, float hy,
                                        float hz, float qx, float qy, float qz) {
  float gx = fmaxf(fmaxf(__fsub_rn(lx, qx), __fsub_rn(qx, hx)), 0.0f);
  float gy = fmaxf(fmaxf(__fsub_rn(ly, qy), __fsub_rn(qy, hy)), 0.0f);
  float gz = fmaxf(fmaxf(__fsub_rn(lz, qz), __fsub_rn(qz, hz)), 0.0f);
  return __fmaf_rn(gz, gz, __fmaf_rn(gx, gx, __fmul_rn(gy, gy)));
}

// Paired FP32 arithmetic (sm_100 and later): two IEEE round-to-nearest
// operations per instruction, so a paired expression gives the same bits as
// the scalar one.
__device__ __forceinline__ unsigned long long f2_pack(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
// d2_box of the four children of a group (same operations, same bits): the
// group's structure-of-arrays lanes pair up as (0, 1) and (2, 3); only the
// max has no paired form
__device__ __forceinline__ void d2_box4(float4 lx, float4 ly, float4 lz, float4 hx, float4 hy, float4 hz,
                                        unsigned long long qx2, unsigned long long qy2, unsigned long long qz2,
                                        float& m0, float& m1, float& m2, float& m3) {
  float a0, a1, a2, a3, b0, b1, b2, b3;
  unsigned long long g01[3], g23[3];
  const float4* lo[3] = {&lx, &ly, &lz};
  const float4* hi[3] = {&hx, &hy, &hz};
  const unsigned long long q2[3] = {qx2, qy2, qz2};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    f2_unpack(f2_sub(f2_pack(lo[a]->x, lo[a]->y), q2[a]), a0, a1);
    f2_unpack(f2_sub(f2_pack(lo[a]->z, lo[a]->w), q2[a]), a2, a3);
    f2_unpack(f2_sub(q2[a], f2_pack(hi[a]->x, hi[a]->y)), b0, b1);
    f2_unpack(f2_sub(q2[a], f2_pack(hi[a]->z, hi[a]->w)), b2, b3);
    g01[a] = f2_pack(fmaxf(fmaxf(a0, b0), 0.0f), fmaxf(fmaxf(a1, b1), 0.0f));
    g23[a] = f2_pack(fmaxf(fmaxf(a2, b2), 0.0f), fmaxf(fmaxf(a3, b3), 0.0f));
  }
  f2_unpack(f2_fma(g01[2], g01[2], f2_fma(g01[0], g01[0], f2_mul(g01[1], g01[1]))), m0, m1);
  f2_unpack(f2_fma(g23[2], g23[2], f2_fma(g23[0], g23[0], f2_mul(g23[1], g23[1]))), m2, m3);
}

// k nearest candidates kept sorted by (d2, cloud index) ascending.
template <int K>
struct KList {
  float d[K];
  int32_t s[K];   // sorted position, -1 = empty
  float r[K];     // record .w (radius)
};

template <int K>
__device__ __forceinline__ void klist_init(KList<K>& L) {
#pragma unroll
  for (int j = 0; j < K; ++j) {
    L.d[j] = __int_as_float(0x7f800000);
    L.s[j] = -1;
    L.r[j] = 0.0f;
  }
}

// (d, s) before (dj, sj)?  Equal distances compare cloud indices (rare path).
__device__ __forceinline__ bool knn_before(float d, int32_t s, float dj, int32_t sj,
                                           const int32_t* __restrict__ perm) {
  if (d < dj) return true;
  if (!(d == dj) || sj < 0) return false;
  return __ldg(perm + s) < __ldg(perm + sj);
}

template <int K>
__device__ __forceinline__ void klist_insert(KList<K>& L, float d, int32_t s, float r,
                                             const int32_t* __restrict__ perm) {
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (knn_before(d, s, L.d[j], L.s[j], perm)) {
      float td = L.d[j];
      int32_t ts = L.s[j];
      float tr = L.r[j];
      L.d[j] = d;
      L.s[j] = s;
      L.r[j] = r;
      d = td;
      s = ts;
      r = tr;
    }
  }
}

// The marcher's 10 nearest, kept sorted by d2 in registers (runs of equal
// d2 put in cloud-index order by order() before they are read), with
// placeholder entries (index -1) last, so the bound is always d[KNN-1].  A
// step starts with restart(): ten placeholders one ulp above the largest
// distance of the previous step's points at the new position (a valid
// bound: those are ten real candidates), so the search prunes with a finite
// bound from the first node and stays exact, and every point it keeps is
// met once.  Radii are not kept here; the step value reads them from the
// records.
//
// Cost.  An insertion is the hot divergent path of the packet walk (about
// 30 per ray step at 20M points), so its common case touches no memory and
// takes no branch: one select pass that slides the new entry into place,
// with all ten comparisons independent of each other (a serial
// compare-and-swap chain would leave the warp waiting on each result).
// Exact d2 ties only matter when one of the tied entries is about to leave
// the set; that case (the 9th and 10th entries equal) takes the ordered
// path, which compares cloud indices.  An earlier form kept the previous
// step's points in the set and re-sorted them; the walk then met each of
// them a second time, and every insertion had to test for duplicates first
// (that form was 6% slower, with 80 more bytes of spills at 64 registers).
struct KSet {
  float d[KNN];
  int32_t s[KNN];   // sorted position, -1 = empty

  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int j = 0; j < KNN; ++j) {
      d[j] = __int_as_float(0x7f800000);
      s[j] = -1;
    }
  }

  __device__ __forceinline__ float worst() const { return d[KNN - 1]; }

  // Candidate (dd, ss) with dd <= worst().  Fast path: dd is strictly
  // below the 10th entry, and the entry it pushes out (the 10th) is strictly
  // above the 9th or a placeholder, so no tie decides what leaves the set;
  // the new entry goes in by d2 alone, after any equal entries, and order()
  // sorts equal entries by cloud index before the set is read.
  __device__ __forceinline__ void consider(float dd, int32_t ss, const int32_t* __restrict__ perm) {
    if (dd < d[KNN - 1] && (d[KNN - 2] < d[KNN - 1] || s[KNN - 2] < 0)) {
#pragma unroll
      for (int j = KNN - 1; j > 0; --j) {
        const bool g = d[j] > dd, gp = d[j - 1] > dd;
        d[j] = g ? (gp ? d[j - 1] : dd) : d[j];
        s[j] = g ? (gp ? s[j - 1] : ss) : s[j];
      }
      const bool g0 = d[0] > dd;
      d[0] = g0 ? dd : d[0];
      s[0] = g0 ? ss : s[0];
      return;
    }
    order(perm);
    consider_ordered(dd, ss, perm);
  }

  // Equal distances present: skip a duplicate, else insert by (d2, cloud index).
  __device__ __forceinline__ void consider_ordered(float dd, int32_t ss, const int32_t* __restrict__ perm) {
    bool dup = false;
#pragma unroll
    for (int j = 0; j < KNN; ++j) dup |= (s[j] == ss);
    if (dup) return;
#pragma unroll
    for (int j = 0; j < KNN; ++j) {
      if (s[j] < 0 || knn_before(dd, ss, d[j], s[j], perm)) {  // placeholders are last
        const float td = d[j];
        const int32_t ts = s[j];
        d[j] = dd;
        s[j] = ss;
        dd = td;
        ss = ts;
      }
    }
  }

  // Sorts runs of equal d2 by cloud index (an insertion pass, taken only
  // when two adjacent real entries have equal d2).
  __device__ __forceinline__ void order(const int32_t* __restrict__ perm) {
    bool tie = false;
#pragma unroll
    for (int j = 0; j + 1 < KNN; ++j) tie |= (d[j] == d[j + 1] && s[j + 1] >= 0);
    if (tie) {
#pragma unroll
      for (int i = 1; i < KNN; ++i) {
#pragma unroll
        for (int j = i; j > 0; --j) {
          if (s[j] >= 0 && knn_before(d[j], s[j], d[j - 1], s[j - 1], perm)) {
            const float td = d[j];
            const int32_t ts = s[j];
            d[j] = d[j - 1];
            s[j] = s[j - 1];
            d[j - 1] = td;
            s[j - 1] = ts;
          }
        }
      }
    }
  }

  // Start of a step.  The previous step's ten points, re-measured at the new
  // position, are ten valid candidates, so the largest of their distances w
  // bounds the new 10th distance.  The set restarts empty, with placeholder
  // entries (index -1) one ulp above w: the walk prunes with that bound from
  // its first node, and the real points it finds (the ten again among them)
  // replace the placeholders.  Restarting empty, rather than keeping the ten
  // in the set, means that no point is met twice in a walk, so the common
  // insertion needs no duplicate test.
  __device__ __forceinline__ void restart(const IndexDev& ix, float qx, float qy, float qz) {
    float w = 0.0f;
    bool full = true;
#pragma unroll
    for (int j = 0; j < KNN; ++j) {
      if (s[j] >= 0) w = fmaxf(w, d2_point(__ldg(ix.rec + s[j]), qx, qy, qz));
      else full = false;
    }
    const float ph = (full && w < __int_as_float(0x7f800000)) ? __int_as_float(__float_as_int(w) + 1)
                                                              : __int_as_float(0x7f800000);
#pragma unroll
    for (int j = 0; j < KNN; ++j) {
      d[j] = ph;
      s[j] = -1;
    }
  }

  // src/ray_marching.cu:280-290: min of sqrtf(d2) - r visiting candidates
  // in ascending (d2, index) order with a strict "<" -- equivalently the
  // minimum value, ties going to the smaller (d2, index).
  __device__ __forceinline__ float step_value(const IndexDev& ix, int32_t* best_s) const {
    float best = __int_as_float(0x7f800000), bd = best;
    int32_t bs = -1;
#pragma unroll
    for (int j = 0; j < KNN; ++j) {
      if (s[j] >= 0) {
        float v = __fsub_rn(__fsqrt_rn(d[j]), __ldg(&ix.rec[s[j]].w));
        bool take = v < best;
        if (!take && v == best)
          take = d[j] < bd || (d[j] == bd && __ldg(ix.perm + s[j]) < __ldg(ix.perm + bs));
        if (take) {
          best = v;
          bd = d[j];
          bs = s[j];
        }
      }
    }
    *best_s = bs;
    return best;
  }
};

__device__ __forceinline__ float list_worst(const KSet& L) { return L.worst(); }
template <int K>
__device__ __forceinline__ float list_worst(const KList<K>& L) { return L.d[K - 1]; }
__device__ __forceinline__ void list_consider(KSet& L, float d, int32_t s, float r, const int32_t* perm) {
  (void)r;
  L.consider(d, s, perm);
}
template <int K>
__device__ __forceinline__ void list_consider(KList<K>& L, float d, int32_t s, float r, const int32_t* perm) {
  klist_insert<K>(L, d, s, r, perm);
}

template <class List>
__device__ __forceinline__ void scan_leaf(const IndexDev& ix, int64_t leaf, float qx, float qy,
                                          float qz, List& L) {
  int64_t start = leaf * ix.leaf;
  int64_t end = start + ix.leaf;
  if (end > ix.n) end = ix.n;
  for (int64_t i = start; i < end; ++i) {
    float4 c = __ldg(ix.rec + i);
    float d = d2_point(c, qx, qy, qz);
    if (d <= list_worst(L)) list_consider(L, d, (int32_t)i, c.w, ix.perm);
  }
}

#define RM_CSWAP(ma, ca, mb, cb)              \
  do {                                        \
    if ((mb) < (ma)) {                        \
      float _tm = (ma); (ma) = (mb); (mb) = _tm; \
      int _tc = (ca); (ca) = (cb); (cb) = _tc;   \
    }                                         \
  } while (0)

// Exact k-NN over the implicit 4-ary tree.  A subtree is expanded whenever
// its box bound is <= the current k-th distance, so equal-distance points
// with a lower index are never skipped.  Returns false only if the stack
// bound was exceeded (cannot happen for depth <= MAX_LEVELS).
// The caller initialises (or seeds) L.
template <class List>
__device__ bool knn_search(const IndexDev& ix, float qx, float qy, float qz, List& L) {
  if (ix.n <= 0) return true;
  uint32_t stk[STACK];
  float stkd[STACK];
  int sp = 0;
  int lvl = 0;
  uint32_t j = 0;
  while (true) {
    const float4* g = ix.groups + (size_t)GROUP_F4 * (size_t)(group_offset(lvl) + j);
    float4 lx = __ldg(g + 0), ly = __ldg(g + 1), lz = __ldg(g + 2);
    float4 hx = __ldg(g + 3), hy = __ldg(g + 4), hz = __ldg(g + 5);
    float m0 = d2_box(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, qx, qy, qz);
    float m1 = d2_box(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, qx, qy, qz);
    float m2 = d2_box(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, qx, qy, qz);
    float m3 = d2_box(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, qx, qy, qz);
    int c0 = 0, c1 = 1, c2 = 2, c3 = 3;
    RM_CSWAP(m0, c0, m1, c1);
    RM_CSWAP(m2, c2, m3, c3);
    RM_CSWAP(m0, c0, m2, c2);
    RM_CSWAP(m1, c1, m3, c3);
    RM_CSWAP(m1, c1, m2, c2);
    uint32_t base = j * 4u;
    if (lvl + 1 == ix.depth) {
      if (m0 <= list_worst(L)) {
        scan_leaf(ix, base + c0, qx, qy, qz, L);
        if (m1 <= list_worst(L)) {
          scan_leaf(ix, base + c1, qx, qy, qz, L);
          if (m2 <= list_worst(L)) {
            scan_leaf(ix, base + c2, qx, qy, qz, L);
            if (m3 <= list_worst(L)) scan_leaf(ix, base + c3, qx, qy, qz, L);
          }
        }
      }
    } else {
      float w = list_worst(L);
      if (sp + 3 > STACK) return false;
      uint32_t code = (uint32_t)(lvl + 1) << 28;
      if (m3 <= w) { stk[sp] = code | (base + c3); stkd[sp] = m3; ++sp; }
      if (m2 <= w) { stk[sp] = code | (base + c2); stkd[sp] = m2; ++sp; }
      if (m1 <= w) { stk[sp] = code | (base + c1); stkd[sp] = m1; ++sp; }
      if (m0 <= w) {
        lvl = lvl + 1;
        j = base + c0;
        continue;
      }
    }
    bool found = false;
    while (sp > 0) {
      --sp;
      if (stkd[sp] <= list_worst(L)) {
        lvl = (int)(stk[sp] >> 28);
        j = stk[sp] & 0x0fffffffu;
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  return true;
}

// Per-warp shared memory of a packet traversal: pending nodes (their boxes
// are re-read from the parent's group and re-tested when popped).
constexpr int PSTACK = 3 * MAX_LEVELS + 4;
// Node expansions one packet walk may take before it gives up and reports
// an error (far above any exact search's need; only a broken bound hits it).
constexpr unsigned PACKET_NODE_BUDGET = 1u << 20;
struct PacketStack {
  uint32_t code[PSTACK];
  float4 rec[32];  // one staged leaf (leaf size <= 32)
};

// Shared memory of the best-first walk: the depth-first stack and staged
// leaf of PacketStack plus the queue's overflow stack, and two event counts
// kept by lane 0 (entries moved to the overflow stack; walks that fell back
// to depth-first order) for the launch statistics.
constexpr int PKT_OVERFLOW = 256;
struct PacketQueue : PacketStack {
  uint32_t over[PKT_OVERFLOW];
  unsigned n_spill;
  unsigned n_dfs;
};

__device__ __forceinline__ void list_consider_unique(KSet& L, float d, int32_t s, float r,
                                                     const int32_t* perm) {
  (void)r;
  L.consider(d, s, perm);
}
template <int K>
__device__ __forceinline__ void list_consider_unique(KList<K>& L, float d, int32_t s, float r,
                                                     const int32_t* perm) {
  bool dup = false;
#pragma unroll
  for (int j = 0; j < K; ++j) dup |= (L.s[j] == s);
  if (!dup) klist_insert<K>(L, d, s, r, perm);
}

#define RM_CSWAP_U(ka, ca, kb, cb)                 \
  do {                                             \
    if ((kb) < (ka)) {                             \
      float _t = (ka); (ka) = (kb); (kb) = _t;     \
      int _c = (ca); (ca) = (cb); (cb) = _c;       \
    }                                              \
  } while (0)

// Warp packet traversal: exact k-NN of every active lane's query with one
// walk of the tree for the whole warp.  A node is expanded when its box lies
// within the current k-th distance of ANY active lane (one OR-reduction of
// 4-bit votes per node), children are visited nearest-first for the leading
// lane, pending nodes wait on a shared-memory stack and are re-tested when
// popped (their boxes re-read from the parent's group), and a leaf's records
// are staged once for the warp (broadcast loads) while every lane updates
// its own list.  Lists may arrive seeded (insertions skip points already
// present).  All 32 lanes call it with warp-uniform control flow; inactive
// lanes only follow along.  Returns false if the stack bound or the node
// budget was hit (neither can happen for depth <= MAX_LEVELS and an exact
// bound).
//
// Nodes are addressed by their group's level-order index G: the children of
// G have groups 4G + 1 + c, and a stack entry holds (level << 28) | G, so no
// level offset is computed on the walk.  Leaves are never pushed: they are
// scanned in order when their parent (a node of level depth-1) is expanded.
template <class List>
__device__ bool packet_knn(const IndexDev& ix, bool active, float qx, float qy, float qz, List& L,
                           PacketStack& ps, unsigned& leaves, unsigned& nodes) {
  const unsigned FULL = 0xffffffffu;
  const float INF = __int_as_float(0x7f800000);
  const int lane = threadIdx.x & 31;
  unsigned act = __ballot_sync(FULL, active);
  if (act == 0 || ix.n <= 0) return true;
  // the visiting order follows one lane: a central pixel of an 8x4 tile
  // (lanes 11, 12, 19, 20) when one is active, whose nearest-first order
  // suits its neighbours better than a corner's
  const unsigned central = act & 0x00181800u;
  const int leader = __ffs(central ? central : act) - 1;
  const uint32_t last_first = (uint32_t)group_offset(ix.depth - 1);  // first group of level depth-1
  const unsigned long long qx2 = f2_pack(qx, qx), qy2 = f2_pack(qy, qy), qz2 = f2_pack(qz, qz);
  int sp = 0;
  int lvl = 0;
  uint32_t G = 0;
  unsigned budget = PACKET_NODE_BUDGET;
  while (true) {
    ++nodes;
    if (--budget == 0) return false;  // self-check: a walk this long means a broken bound
    const float4* g = ix.groups + (size_t)GROUP_F4 * G;
    float m0, m1, m2, m3;
    {
      float4 lx = __ldg(g + 0), ly = __ldg(g + 1), lz = __ldg(g + 2);
      float4 hx = __ldg(g + 3), hy = __ldg(g + 4), hz = __ldg(g + 5);
      d2_box4(lx, ly, lz, hx, hy, hz, qx2, qy2, qz2, m0, m1, m2, m3);
    }
    // needed children: one OR-reduction of every active lane's 4-bit vote
    // (idle lanes do not vote: their bound may be +inf, and inf <= inf)
    const float w = list_worst(L);
    unsigned mine = 0;
    if (active) mine = (m0 <= w ? 1u : 0u) | (m1 <= w ? 2u : 0u) | (m2 <= w ? 4u : 0u) | (m3 <= w ? 8u : 0u);
    const unsigned needm = __reduce_or_sync(FULL, mine);
    if (needm != 0) {
      // visiting order (2 bits per position, nearest first for the leading
      // lane); with one needed child any order will do
      unsigned order = 0xE4u;  // 0, 1, 2, 3
      if (needm & (needm - 1u)) {
        float k0 = m0, k1 = m1, k2 = m2, k3 = m3;
        int o0 = 0, o1 = 1, o2 = 2, o3 = 3;
        RM_CSWAP_U(k0, o0, k1, o1);
        RM_CSWAP_U(k2, o2, k3, o3);
        RM_CSWAP_U(k0, o0, k2, o2);
        RM_CSWAP_U(k1, o1, k3, o3);
        RM_CSWAP_U(k1, o1, k2, o2);
        order = __shfl_sync(FULL, (unsigned)o0 | ((unsigned)o1 << 2) | ((unsigned)o2 << 4) | ((unsigned)o3 << 6),
                            leader);
      }
      if (lvl + 1 == ix.depth) {
        const uint32_t lbase = (G - last_first) * 4u;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int c = (int)((order >> (2 * t)) & 3u);
          if (!(needm & (1u << c))) continue;
          // bounds may have shrunk while scanning nearer leaves
          const float mc = c == 0 ? m0 : c == 1 ? m1 : c == 2 ? m2 : m3;
          if (!__ballot_sync(FULL, active && mc <= list_worst(L))) continue;
          const int64_t start = (int64_t)(lbase + c) * ix.leaf;
          const int cnt = (int)min((int64_t)ix.leaf, ix.n - start);
          ++leaves;
          // one coalesced load of the leaf into shared memory, then broadcast
          // reads (one point per iteration: the insertion is inlined at this
          // single site, and unrolling it costs more in instruction fetch
          // than it saves)
          __syncwarp();
          if (lane < cnt) ps.rec[lane] = __ldg(ix.rec + start + lane);
          __syncwarp();
          if (active) {
            for (int k = 0; k < cnt; ++k) {
              const float4 cr = ps.rec[k];
              const float d = d2_point(cr, qx, qy, qz);
              if (d <= list_worst(L)) list_consider_unique(L, d, (int32_t)(start + k), cr.w, ix.perm);
            }
          }
        }
      } else {
        // descend into the nearest needed child; lanes 0-3 push the others
        // (order position t by lane t), farthest deepest so the nearest pops first
        unsigned om = 0;  // bit t: the child at order position t is needed
#pragma unroll
        for (int t = 0; t < 4; ++t) om |= ((needm >> ((order >> (2 * t)) & 3u)) & 1u) << t;
        const int tf = __ffs(om) - 1;
        const unsigned rest = om & (om - 1u);
        if (sp + 3 > PSTACK) return false;
        const uint32_t child0 = 4u * G + 1u;
        if (lane < 4 && ((rest >> lane) & 1u)) {
          const int slot = sp + __popc(rest >> (lane + 1));
          ps.code[slot] = ((uint32_t)(lvl + 1) << 28) | (child0 + ((order >> (2 * lane)) & 3u));
        }
        sp += __popc(rest);
        __syncwarp();
        lvl = lvl + 1;
        G = child0 + ((order >> (2 * tf)) & 3u);
        continue;
      }
    }
    bool found = false;
    while (sp > 0) {
      --sp;
      const uint32_t code = ps.code[sp];
      const int plvl = (int)(code >> 28);
      const uint32_t pG = code & 0x0fffffffu;
      // the node's box: lane (pG - 1) & 3 of its parent's group (pG - 1) >> 2
      const float* pg = reinterpret_cast<const float*>(ix.groups + (size_t)GROUP_F4 * ((pG - 1u) >> 2));
      const int c = (int)((pG - 1u) & 3u);
      float md = INF;
      if (active)
        md = d2_box(__ldg(pg + 0 + c), __ldg(pg + 4 + c), __ldg(pg + 8 + c), __ldg(pg + 12 + c),
                    __ldg(pg + 16 + c), __ldg(pg + 20 + c), qx, qy, qz);
      if (__ballot_sync(FULL, active && md <= list_worst(L))) {
        lvl = plvl;
        G = pG;
        found = true;
        break;
      }
    }
    __syncwarp();
    if (!found) break;
  }
  return true;
}

// Best-first form of packet_knn for the marcher.  The depth-first walk
// finishes the leading lane's subtree before anything else, so lanes whose
// nearest points lie in another subtree keep loose bounds (and so want
// most leaves) for much of the walk.  Here pending nodes wait in a priority
// queue keyed by the leading lane's box distance, and the walk always
// continues with the nearest one; the leaves of a node at level depth-1
// are scanned when it is expanded.  A CPU simulation of both walks on
// recorded warp steps gave about 20% fewer leaves and 12% fewer nodes.
// The queue is 32 entries in registers (lane i holds the i-th nearest);
// the farthest entry of a full queue moves to an overflow stack in shared
// memory, and if that fills as well the walk continues depth-first on the
// bounded stack from then on.  Every taken node's children are tested
// against the bounds of that moment, so the result is exact whatever the
// order.
template <class List>
__device__ bool packet_knn_bf(const IndexDev& ix, bool active, float qx, float qy, float qz, List& L,
                              PacketQueue& ps, unsigned& leaves, unsigned& nodes) {
  const unsigned FULL = 0xffffffffu;
  const float INF = __int_as_float(0x7f800000);
  const int lane = threadIdx.x & 31;
  unsigned act = __ballot_sync(FULL, active);
  if (act == 0 || ix.n <= 0) return true;
  // the visiting order follows one lane: a central pixel of an 8x4 tile
  // (lanes 11, 12, 19, 20) when one is active, whose nearest-first order
  // suits its neighbours better than a corner's
  const unsigned central = act & 0x00181800u;
  const int leader = __ffs(central ? central : act) - 1;
  const uint32_t last_first = (uint32_t)group_offset(ix.depth - 1);  // first group of level depth-1
  const unsigned long long qx2 = f2_pack(qx, qx), qy2 = f2_pack(qy, qy), qz2 = f2_pack(qz, qz);
  int sp = 0;     // depth-first stack (ps.code from the bottom), used once `dfs` is set
  int fsp = 0;    // far entries spilled at the switch (ps.code from the top), taken last
  int osp = 0;    // overflow stack (ps.over)
  int qn = 0;     // register queue: lane i holds the i-th nearest pending node
  float qkey = INF;
  uint32_t qcode = 0;
  bool dfs = false;
  // queue insert (warp-uniform key and code); the farthest entry of a full
  // queue moves to the overflow stack, and a full overflow stack switches
  // the walk to depth-first mode on the bounded stack.  Entries spilled in
  // the switching expansion (at most four: no queue insert happens after
  // the switch) wait at the top of that stack and are taken last, after
  // the queue and the overflow, so that far subtrees are not walked while
  // the bounds are still loose.
  auto spill = [&](uint32_t code) {
    if (!dfs && osp < PKT_OVERFLOW) {
      if (lane == 0) {
        ps.over[osp] = code;
        ++ps.n_spill;
      }
      ++osp;
    } else {
      if (!dfs && lane == 0) ++ps.n_dfs;
      dfs = true;
      if (sp + fsp < PSTACK && lane == 0) ps.code[PSTACK - 1 - fsp] = code;
      ++fsp;
    }
  };
  auto qpush = [&](float key, uint32_t code) {
    const int pos = __popc(__ballot_sync(FULL, lane < qn && qkey <= key));
    if (qn == 32) {
      if (pos == 32) {
        spill(code);
        return;
      }
      spill(__shfl_sync(FULL, qcode, 31));
    } else {
      ++qn;
    }
    const float ku = __shfl_up_sync(FULL, qkey, 1);
    const uint32_t cu = __shfl_up_sync(FULL, qcode, 1);
    if (lane > pos) {
      qkey = ku;
      qcode = cu;
    }
    if (lane == pos) {
      qkey = key;
      qcode = code;
    }
  };
  int lvl = 0;
  uint32_t G = 0;
  const unsigned nodes0 = nodes;
  while (true) {
    ++nodes;
    if (nodes - nodes0 >= PACKET_NODE_BUDGET) return false;  // self-check: a walk this long means a broken bound
    const float4* g = ix.groups + (size_t)GROUP_F4 * G;
    float m0, m1, m2, m3;
    {
      float4 lx = __ldg(g + 0), ly = __ldg(g + 1), lz = __ldg(g + 2);
      float4 hx = __ldg(g + 3), hy = __ldg(g + 4), hz = __ldg(g + 5);
      d2_box4(lx, ly, lz, hx, hy, hz, qx2, qy2, qz2, m0, m1, m2, m3);
    }
    // needed children: one OR-reduction of every active lane's 4-bit vote
    // (idle lanes do not vote: their bound may be +inf, and inf <= inf)
    const float w = list_worst(L);
    unsigned mine = 0;
    if (active) mine = (m0 <= w ? 1u : 0u) | (m1 <= w ? 2u : 0u) | (m2 <= w ? 4u : 0u) | (m3 <= w ? 8u : 0u);
    const unsigned needm = __reduce_or_sync(FULL, mine);
    if (needm != 0 && lvl + 1 != ix.depth && !dfs) {
      // Inner node, best-first.  Keys are the leading lane's box distances:
      // the walk descends into the nearest needed child unless a queued node
      // is nearer still, and queues the other needed children (the queue
      // keeps them in key order, so no ordering network is needed here).
      const uint32_t child0 = 4u * G + 1u;
      const uint32_t lcode = (uint32_t)(lvl + 1) << 28;
      if (!(needm & (needm - 1u))) {
        // one child (about 35% of expansions): one shuffle
        const int c = __ffs(needm) - 1;
        const float kc = __shfl_sync(FULL, c == 0 ? m0 : c == 1 ? m1 : c == 2 ? m2 : m3, leader);
        if (qn == 0 || kc <= __shfl_sync(FULL, qkey, 0)) {
          lvl = lvl + 1;
          G = child0 + (uint32_t)c;
          continue;
        }
        qpush(kc, lcode | (child0 + (uint32_t)c));
      } else {
        const float k0 = __shfl_sync(FULL, m0, leader), k1 = __shfl_sync(FULL, m1, leader);
        const float k2 = __shfl_sync(FULL, m2, leader), k3 = __shfl_sync(FULL, m3, leader);
        const float e0 = (needm & 1u) ? k0 : INF, e1 = (needm & 2u) ? k1 : INF;
        const float e2 = (needm & 4u) ? k2 : INF, e3 = (needm & 8u) ? k3 : INF;
        const int c01 = e1 < e0 ? 1 : 0, c23 = e3 < e2 ? 3 : 2;
        const float k01 = fminf(e0, e1), k23 = fminf(e2, e3);
        const int cf = k23 < k01 ? c23 : c01;  // nearest needed child, ties to the lower index
        const bool down = qn == 0 || fminf(k01, k23) <= __shfl_sync(FULL, qkey, 0);
        const unsigned topush = down ? (needm & ~(1u << cf)) : needm;
        if (topush & 1u) qpush(k0, lcode | child0);
        if (topush & 2u) qpush(k1, lcode | (child0 + 1u));
        if (topush & 4u) qpush(k2, lcode | (child0 + 2u));
        if (topush & 8u) qpush(k3, lcode | (child0 + 3u));
        if (down) {
          if (sp + fsp > PSTACK) return false;
          __syncwarp();
          lvl = lvl + 1;
          G = child0 + (uint32_t)cf;
          continue;
        }
      }
      if (sp + fsp > PSTACK) return false;
    } else if (needm != 0) {
      // Leaf level (its leaves are scanned now), or the depth-first fallback.
      // Visiting order (2 bits per position, nearest first for the leading
      // lane); with one needed child any order will do.
      unsigned order = 0xE4u;  // 0, 1, 2, 3
      if (needm & (needm - 1u)) {
        float k0 = m0, k1 = m1, k2 = m2, k3 = m3;
        int o0 = 0, o1 = 1, o2 = 2, o3 = 3;
        RM_CSWAP_U(k0, o0, k1, o1);
        RM_CSWAP_U(k2, o2, k3, o3);
        RM_CSWAP_U(k0, o0, k2, o2);
        RM_CSWAP_U(k1, o1, k3, o3);
        RM_CSWAP_U(k1, o1, k2, o2);
        order = __shfl_sync(FULL, (unsigned)o0 | ((unsigned)o1 << 2) | ((unsigned)o2 << 4) | ((unsigned)o3 << 6),
                            leader);
      }
      if (lvl + 1 == ix.depth) {
        const uint32_t lbase = (G - last_first) * 4u;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int c = (int)((order >> (2 * t)) & 3u);
          if (!(needm & (1u << c))) continue;
          // bounds may have shrunk while scanning nearer leaves
          const float mc = c == 0 ? m0 : c == 1 ? m1 : c == 2 ? m2 : m3;
          if (!__ballot_sync(FULL, active && mc <= list_worst(L))) continue;
          const int64_t start = (int64_t)(lbase + c) * ix.leaf;
          const int cnt = (int)min((int64_t)ix.leaf, ix.n - start);
          ++leaves;
          // one coalesced load of the leaf into shared memory, then broadcast
          // reads, two points per iteration: their distances are independent
          // (twice the work between dependent instructions), while the
          // insertion stays inlined at one site, in a two-pass loop that only
          // runs when one of the two is within the bound (unrolling the
          // insertion as well costs more in instruction fetch than it saves;
          // two points per iteration measured +2.8%)
          __syncwarp();
          if (lane < cnt) ps.rec[lane] = __ldg(ix.rec + start + lane);
          __syncwarp();
          if (active) {
            for (int k = 0; k < cnt; k += 2) {
              const float4 ca = ps.rec[k], cb = ps.rec[k + 1];  // rec has 32 slots; cb unused past cnt
              const float da = d2_point(ca, qx, qy, qz);
              const float db = k + 1 < cnt ? d2_point(cb, qx, qy, qz) : INF;
              if (fminf(da, db) <= list_worst(L)) {
#pragma unroll 1
                for (int j = 0; j < 2; ++j) {
                  const float dj = j ? db : da;
                  if (dj <= list_worst(L)) list_consider_unique(L, dj, (int32_t)(start + k + j), 0.0f, ix.perm);
                }
              }
            }
          }
        }
      } else {
        unsigned om = 0;  // bit t: the child at order position t is needed
#pragma unroll
        for (int t = 0; t < 4; ++t) om |= ((needm >> ((order >> (2 * t)) & 3u)) & 1u) << t;
        const int tf = __ffs(om) - 1;
        const unsigned rest = om & (om - 1u);
        const uint32_t child0 = 4u * G + 1u;
        const uint32_t lcode = (uint32_t)(lvl + 1) << 28;
        if (dfs) {
          // depth-first: descend into the nearest needed child; lanes 0-3
          // push the others, farthest deepest so the nearest pops first
          if (sp + fsp + 3 > PSTACK) return false;
          if (lane < 4 && ((rest >> lane) & 1u)) {
            const int slot = sp + __popc(rest >> (lane + 1));
            ps.code[slot] = lcode | (child0 + ((order >> (2 * lane)) & 3u));
          }
          sp += __popc(rest);
          __syncwarp();
          lvl = lvl + 1;
          G = child0 + ((order >> (2 * tf)) & 3u);
          continue;
        }
      }
    }
    bool found = false;
    __syncwarp();
    while (true) {
      uint32_t code;
      if (sp > 0) {
        --sp;
        code = ps.code[sp];
      } else if (qn > 0) {
        code = __shfl_sync(FULL, qcode, 0);
        qkey = __shfl_down_sync(FULL, qkey, 1);
        qcode = __shfl_down_sync(FULL, qcode, 1);
        --qn;
      } else if (osp > 0) {
        --osp;
        code = ps.over[osp];
        // Entries on the overflow stack were the farthest of a full queue,
        // and by the time they are taken the bounds have shrunk: about 89%
        // of them are no longer needed (20M-point workload).  Unlike a
        // queue entry (87% still needed when taken), such a node is worth
        // re-testing before its expansion: its box is lane (G - 1) & 3 of
        // its parent's group (about 14 fewer expansions per warp step, +1%).
        const uint32_t pG = code & 0x0fffffffu;
        const float* pg = reinterpret_cast<const float*>(ix.groups + (size_t)GROUP_F4 * ((pG - 1u) >> 2));
        const int c = (int)((pG - 1u) & 3u);
        float md = INF;
        if (active)
          md = d2_box(__ldg(pg + 0 + c), __ldg(pg + 4 + c), __ldg(pg + 8 + c), __ldg(pg + 12 + c),
                      __ldg(pg + 16 + c), __ldg(pg + 20 + c), qx, qy, qz);
        if (!__ballot_sync(FULL, active && md <= list_worst(L))) continue;
      } else if (fsp > 0) {
        --fsp;
        code = ps.code[PSTACK - 1 - fsp];
      } else {
        break;
      }
      // no re-test of the node's own box here: its expansion tests its
      // children against the current bounds, and a child's box lies inside
      // its parent's, so a node that is no longer needed yields no needed
      // child (one dependent load fewer per taken node, measured +1.2%)
      lvl = (int)(code >> 28);
      G = code & 0x0fffffffu;
      found = true;
      break;
    }
    __syncwarp();
    if (!found) break;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Camera rays, src/ray_marching.cu:70-79.

struct Ray {
  float ox, oy, oz;
  float dx, dy, dz;
  float t_near, t_far;
};

// pane = (float)W / (2 * tanf(0.5 * fov)), evaluated on the device as the
// reference's render kernel does (src/ray_marching.cu:74).
__device__ __forceinline__ float view_pane(int width, float fov) {
  return __fdiv_rn((float)width, __fmul_rn(2.0f, tanf(__fmul_rn(0.5f, fov))));
}

// m: column-major cam-to-world (column c at m[4c..4c+3]).
__device__ __forceinline__ Ray make_ray(const float* m, int width, int height, float pane, int x,
                                        int y) {
  Ray r;
  float ux = __fdiv_rn(__fsub_rn(__fmul_rn(2.0f, (float)x), (float)width), 2.0f);
  float uy = __fdiv_rn(__fsub_rn(__fmul_rn(2.0f, (float)y), (float)height), 2.0f);
  float uz = -pane;
  float v[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float a = __fmaf_rn(m[0 + i], ux, __fmul_rn(m[4 + i], uy));
    float b = __fmaf_rn(m[8 + i], uz, __fmul_rn(m[12 + i], 0.0f));
    v[i] = __fadd_rn(a, b);
  }
  float len2 = __fadd_rn(__fmaf_rn(v[0], v[0], __fmul_rn(v[1], v[1])),
                         __fmaf_rn(v[2], v[2], __fmul_rn(v[3], v[3])));
  float inv = __fdiv_rn(1.0f, __fsqrt_rn(len2));
  r.dx = __fmul_rn(v[0], inv);
  r.dy = __fmul_rn(v[1], inv);
  r.dz = __fmul_rn(v[2], inv);
  float cx = -m[8], cy = -m[9], cz = -m[10];
  float dd = __fmaf_rn(cz, r.dz, __fmaf_rn(cx, r.dx, __fmul_rn(cy, r.dy)));
  r.t_far = __fdiv_rn(ZFAR, dd);
  r.t_near = __fdiv_rn(ZNEAR, dd);
  r.ox = m[12];
  r.oy = m[13];
  r.oz = m[14];
  return r;
}

}  // namespace rm
