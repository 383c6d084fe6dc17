// ref_driver.cpp -- drives the reference's vendored FLANN CPU kd-tree
// (third_party/flann/algorithms/kdtree_index.h, exact when searched with
// FLANN_CHECKS_UNLIMITED, kdtree_index.h:227-238) to produce golden vectors
// for the oracle.  TEST INFRASTRUCTURE: built by oracle/Makefile.ref into
// oracle/_ref/ from the sources under the reference tree, run only by
// tests/golden/make_golden.py in the container that has the reference.
//
// Modes (all files raw little-endian):
//   knn   <pts.f32 n*3> <n> <queries.f32 m*3> <m> <k> <out.i32 m*k> <out.f32 m*k>
//         FLANN's own answer (its CPU L2 evaluates ((dx^2 + dy^2) + dz^2)).
//   radii <pts.f32 n*3> <n> <out_r.f32 n> <out_nn.i32 n>
//         the reference's radii (main.cu:107-113) with the GPU's squared
//         distance: FLANN's 16 nearest, re-ranked by fma(dz,dz,fma(dx,dx,dy*dy))
//         and index, second entry.  FLANN's CPU "exact" search adds each
//         split's axis gap to the parent's bound even when an ancestor split
//         on the same axis (kdtree_index.h:656-662), which over-estimates the
//         bound and can prune true neighbours; asking for many more
//         candidates than needed and re-ranking hides that.
//
// FLANN's CPU search is not exact even with FLANN_CHECKS_UNLIMITED (see the
// radii note), so the marcher is pinned by brute force in the tests rather
// than by a FLANN-driven loop.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "flann/flann.hpp"

namespace {

template <class T>
std::vector<T> read_file(const char* path, size_t count) {
  std::vector<T> v(count);
  FILE* f = fopen(path, "rb");
  if (!f || fread(v.data(), sizeof(T), count, f) != count) {
    fprintf(stderr, "cannot read %zu items from %s\n", count, path);
    exit(2);
  }
  fclose(f);
  return v;
}

template <class T>
void write_file(const char* path, const T* data, size_t count) {
  FILE* f = fopen(path, "wb");
  if (!f || fwrite(data, sizeof(T), count, f) != count) {
    fprintf(stderr, "cannot write %s\n", path);
    exit(2);
  }
  fclose(f);
}

float d2_gpu(const float* c, const float* q) {
  float dx = c[0] - q[0], dy = c[1] - q[1], dz = c[2] - q[2];
  return std::fma(dz, dz, std::fma(dx, dx, dy * dy));
}

struct Knn {
  flann::Matrix<float> data;
  flann::KDTreeIndex<flann::L2<float>>* index;
  const float* pts;
  size_t n;
  Knn(float* p, size_t n_) : data(p, n_, 3), pts(p), n(n_) {
    index = new flann::KDTreeIndex<flann::L2<float>>(data, flann::KDTreeIndexParams(1));
    index->buildIndex();
  }
  // FLANN's k nearest of q, re-ranked by the GPU distance and index.
  void query_exact(const float* q, int k, int extra, int* oi, float* od) const {
    int kk = (int)std::min<size_t>(k + extra, n);
    std::vector<int> idx(kk);
    std::vector<float> dd(kk);
    flann::Matrix<float> qm(const_cast<float*>(q), 1, 3);
    flann::Matrix<int> im(idx.data(), 1, kk);
    flann::Matrix<float> dm(dd.data(), 1, kk);
    flann::SearchParams sp(flann::FLANN_CHECKS_UNLIMITED, 0.0f, true);
    index->knnSearch(qm, im, dm, kk, sp);
    std::vector<std::pair<float, int>> c;
    for (int j = 0; j < kk; ++j)
      if (idx[j] >= 0) c.push_back({d2_gpu(pts + 3 * (size_t)idx[j], q), idx[j]});
    std::sort(c.begin(), c.end());
    for (int j = 0; j < k; ++j) {
      if (j < (int)c.size()) {
        oi[j] = c[j].second;
        od[j] = c[j].first;
      } else {
        oi[j] = -1;
        od[j] = INFINITY;
      }
    }
  }
};

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) return 1;
  std::string mode = argv[1];
  if (mode == "knn" && argc == 9) {
    size_t n = atoll(argv[3]), m = atoll(argv[5]);
    int k = atoi(argv[6]);
    auto pts = read_file<float>(argv[2], n * 3);
    auto qs = read_file<float>(argv[4], m * 3);
    flann::Matrix<float> data(pts.data(), n, 3);
    flann::KDTreeIndex<flann::L2<float>> index(data, flann::KDTreeIndexParams(1));
    index.buildIndex();
    std::vector<int> idx(m * k);
    std::vector<float> dd(m * k);
    flann::Matrix<float> qm(qs.data(), m, 3);
    flann::Matrix<int> im(idx.data(), m, k);
    flann::Matrix<float> dm(dd.data(), m, k);
    flann::SearchParams sp(flann::FLANN_CHECKS_UNLIMITED, 0.0f, true);
    index.knnSearch(qm, im, dm, k, sp);
    write_file(argv[7], idx.data(), idx.size());
    write_file(argv[8], dd.data(), dd.size());
    return 0;
  }
  if (mode == "radii" && argc == 6) {
    size_t n = atoll(argv[3]);
    auto pts = read_file<float>(argv[2], n * 3);
    Knn knn(pts.data(), n);
    std::vector<float> r(n);
    std::vector<int> nn(n);
    for (size_t i = 0; i < n; ++i) {
      int oi[2];
      float od[2];
      knn.query_exact(pts.data() + 3 * i, 2, 14, oi, od);
      r[i] = std::sqrt(od[1]);
      nn[i] = oi[1];
    }
    write_file(argv[4], r.data(), n);
    write_file(argv[5], nn.data(), n);
    return 0;
  }
  fprintf(stderr, "usage: ref_driver knn|radii ...\n");
  return 1;
}
