// marcher_main.cpp -- `marcher.bin`, the command-line driver over the C ABI
// (replaces the reference's main.cu:56-275 for the headless path).
//
// Same flags and meaning (main.cu:61-70, README.md:19-31):
//   -f,--file PLY  -m,--matrices JSON  -o,--output_path DIR  -s,--max_points N
//   -r,--max_radius R (default 0.1)  -d,--headless  -p,--precompute-radii
//   -i,--ignore_existing
// plus two additions that do not change the default behaviour:
//   --batch      render every pending view in one batched launch
//   --autotune   tune the batched launch on the pending views first
// Same files: <ply>.kdtree.radii cache; per view <o>/<parent>/<name> colour
// PNG, <..._depth..> 8-bit depth PNG and its .npy; ".<name>.lock" files held
// with POSIX record locks (what boost::interprocess::file_lock takes on
// Linux) so several processes can share one matrices file.  Same stdout
// lines.  The interactive GLFW window (main.cu:235-267) needs a graphics
// stack that these hosts do not have; without -d the driver says so.
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <memory>
#include <iostream>
#include <numeric>
#include <random>
#include <regex>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "io.hpp"
#include "rm.h"

namespace fs = std::filesystem;
using std::cout;
using std::endl;
using std::string;

namespace {

struct Args {
  string file, matrices, output;
  int max_points = -1;
  float max_radius = 0.1f;
  bool headless = false, precompute = false, ignore_existing = false, batch = false, autotune = false;
};

void usage() {
  cout << "Pointcloud Renderer\nUsage: marcher.bin [OPTIONS]\n\nOptions:\n"
          "  -h,--help                   Print this help message and exit\n"
          "  -f,--file TEXT              Path to PLY pointcloud to render\n"
          "  -m,--matrices TEXT          Path to view matrices json for which to render pointcloud in case of headless rendering\n"
          "  -o,--output_path TEXT       Path where to store renders in case of headless rendering\n"
          "  -s,--max_points INT         Take exact number of points from the PLY file\n"
          "  -r,--max_radius FLOAT       Filter possible outliers in radii file by settings max radius\n"
          "  -d,--headless               Run headlessly without a window\n"
          "  -p,--precompute-radii       Precompute radii even if already precomputed\n"
          "  -i,--ignore_existing        Ignore existing renders and forcefully rewrite them\n"
          "  --batch                     Render all pending views in one batched launch\n"
          "  --autotune                  Tune the batched launch on the pending views first\n";
}

bool parse_args(int argc, char** argv, Args& a) {
  for (int i = 1; i < argc; ++i) {
    string s = argv[i];
    auto value = [&](const char* name) -> string {
      if (i + 1 >= argc) throw std::runtime_error(string(name) + " needs a value");
      return argv[++i];
    };
    if (s == "-h" || s == "--help") { usage(); exit(0); }
    else if (s == "-f" || s == "--file") a.file = value("--file");
    else if (s == "-m" || s == "--matrices") a.matrices = value("--matrices");
    else if (s == "-o" || s == "--output_path") a.output = value("--output_path");
    else if (s == "-s" || s == "--max_points") a.max_points = std::stoi(value("--max_points"));
    else if (s == "-r" || s == "--max_radius") a.max_radius = std::stof(value("--max_radius"));
    else if (s == "-d" || s == "--headless") a.headless = true;
    else if (s == "-p" || s == "--precompute-radii") a.precompute = true;
    else if (s == "-i" || s == "--ignore_existing") a.ignore_existing = true;
    else if (s == "--batch") a.batch = true;
    else if (s == "--autotune") a.autotune = true;
    else {
      std::cerr << "The following argument was not expected: " << s << "\nRun with --help for more information." << endl;
      return false;
    }
  }
  return true;
}

void check(rm_ctx* ctx, rm_status s, const char* what) {
  if (s != RM_OK) throw std::runtime_error(string(what) + ": " + rm_last_error(ctx));
}

// Advisory POSIX record lock on the whole file, held while the fd is open.
struct FileLock {
  int fd = -1;
  FileLock() = default;
  FileLock(const FileLock&) = delete;  // one owner per descriptor
  FileLock& operator=(const FileLock&) = delete;
  bool try_lock(const fs::path& p) {
    fd = ::open(p.c_str(), O_RDWR | O_CREAT, 0644);
    if (fd < 0) return false;
    struct flock fl;
    memset(&fl, 0, sizeof(fl));
    fl.l_type = F_WRLCK;
    fl.l_whence = SEEK_SET;
    if (fcntl(fd, F_SETLK, &fl) != 0) {
      ::close(fd);
      fd = -1;
      return false;
    }
    return true;
  }
  void unlock() {
    if (fd >= 0) {
      struct flock fl;
      memset(&fl, 0, sizeof(fl));
      fl.l_type = F_UNLCK;
      fl.l_whence = SEEK_SET;
      fcntl(fd, F_SETLK, &fl);
      ::close(fd);
      fd = -1;
    }
  }
  ~FileLock() { unlock(); }
};

struct Pending {
  fs::path out, depth_out, lock_path;
  rm_view view;
  std::unique_ptr<FileLock> lock;
};

// Writes one view's files.  `threads`: how many row slices each PNG is
// deflated in at once (the per-view mode gives one view all host cores; the
// batch mode already writes several views at a time, one core each).
void save_outputs(const Pending& p, const std::vector<float>& rgbd, int threads) {
  int w = p.view.width, h = p.view.height;
  std::vector<uint8_t> png;
  rmio::encode_colour_rgba8(w, h, rgbd.data(), png);
  rmio::write_png(p.out.string(), w, h, 4, png.data(), threads);
  std::vector<uint8_t> dpng;
  std::vector<float> depth;
  rmio::encode_depth_u8(w, h, rgbd.data(), dpng, depth);
  rmio::write_npy_f32(p.depth_out.string() + ".npy", h, w, depth.data());
  rmio::write_png(p.depth_out.string(), w, h, 1, dpng.data(), threads);
}

int run(const Args& a) {
  auto output = fs::path(a.output);
  rmio::Cloud cloud = rmio::load_ply(a.file);
  size_t n_all = cloud.size();
  // main.cu:75-87: optional subsample, std::mt19937(42) + std::shuffle
  std::vector<int> max_points_indices(n_all);
  if (a.max_points > 0 && (size_t)a.max_points < n_all) {
    std::iota(max_points_indices.begin(), max_points_indices.end(), 0);
    std::mt19937 g(42);
    std::shuffle(max_points_indices.begin(), max_points_indices.end(), g);
    rmio::Cloud sub;
    sub.xyz.resize(3 * (size_t)a.max_points);
    sub.rgb.resize(3 * (size_t)a.max_points);
    for (int ax = 0; ax < a.max_points; ++ax) {
      memcpy(&sub.xyz[3 * (size_t)ax], &cloud.xyz[3 * (size_t)max_points_indices[ax]], 12);
      memcpy(&sub.rgb[3 * (size_t)ax], &cloud.rgb[3 * (size_t)max_points_indices[ax]], 3);
    }
    cloud = std::move(sub);
  }
  size_t n = cloud.size();
  cout << "Number of points: " << n << endl;

  rm_config cfg;
  rm_config_default(&cfg);
  rm_ctx* ctx = nullptr;
  if (rm_ctx_create(&cfg, &ctx) != RM_OK) throw std::runtime_error("cannot create a CUDA context");
  struct Guard {
    rm_ctx* c;
    ~Guard() { rm_ctx_destroy(c); }
  } guard{ctx};
  check(ctx, rm_cloud_set(ctx, cloud.xyz.data(), 3, cloud.rgb.data(), (int64_t)n, RM_HOST), "upload");
  check(ctx, rm_index_build(ctx), "index build");

  auto radii_path = fs::path(a.file + ".kdtree.radii");
  if (!fs::exists(radii_path) || a.precompute) {
    cout << "Precomputing radii..." << endl;
    std::vector<float> radii(n);
    check(ctx, rm_radii_compute(ctx, a.max_radius, radii.data(), nullptr, RM_HOST), "radii");
    rmio::write_radii_archive(a.file + ".kdtree.radii", radii);
  } else {
    cout << "Using precomputed radii..." << endl;
    std::vector<float> radii_host = rmio::read_radii_archive(radii_path.string());
    // main.cu:128-134 re-indexes the cache only when the point count equals
    // -s (for a full-size cache read with a subsample); kept as is
    if ((size_t)a.max_points == n) {
      std::vector<float> r_h(a.max_points);
      for (int ax = 0; ax < a.max_points; ++ax) {
        size_t src = (size_t)max_points_indices[ax];
        if (src >= radii_host.size()) throw std::runtime_error("The radii file '" + radii_path.string() + "' is too short for -s");
        r_h[ax] = radii_host[src];
      }
      radii_host = r_h;
    }
    if (radii_host.size() != n) {
      throw std::runtime_error("The radii file '" + radii_path.string() +
                               "' does not contain the same number of points as PLY file '" + a.file + "'.");
    }
    check(ctx, rm_radii_set(ctx, radii_host.data(), (int64_t)n, a.max_radius, RM_HOST), "radii");
  }

  if (!a.headless) {
    std::cerr << "Interactive window mode needs an OpenGL window, which is unavailable here; run with -d." << endl;
    return EXIT_FAILURE;
  }
  if (a.matrices.empty()) {
    cout << "The matrix file '" << a.matrices << "' was not found." << endl;
    return EXIT_SUCCESS;
  }
  rmio::Json j;
  {
    std::ifstream probe(a.matrices);
    if (!probe.good()) {
      cout << "Error opening matrix file" << endl;
      return EXIT_SUCCESS;
    }
  }
  cout << "Matrices loaded." << endl;
  j = rmio::load_json(a.matrices);

  std::vector<Pending> pending;
  auto process = [&](const string& target, const rmio::Json& params) {
    auto path = fs::path(target);
    auto last_but_one_segment = *(--(--path.end()));
    auto last_segment = *(--path.end());
    Pending p;
    p.out = output / last_but_one_segment / last_segment;
    p.depth_out = output / last_but_one_segment / std::regex_replace(last_segment.string(), std::regex("_color"), "_depth");
    p.lock_path = output / last_but_one_segment / ("." + last_segment.string() + ".lock");
    if (!fs::exists(output)) fs::create_directory(output);
    if (!fs::exists(output / last_but_one_segment)) fs::create_directory(output / last_but_one_segment);
    if (!a.ignore_existing && fs::exists(p.out)) {
      cout << fs::canonical(fs::absolute(p.out)) << ": ALREADY EXISTS" << endl;
      return;
    }
    { std::ofstream touch{p.lock_path}; }
    p.lock = std::make_unique<FileLock>();
    if (!p.lock->try_lock(p.lock_path)) {
      cout << fs::absolute(p.out) << ": ALREADY LOCKED" << endl;
      return;
    }
    cout << fs::absolute(p.out) << ": LOCKING" << endl;
    float pose[16], K[16];
    rmio::json_mat4(params.at("camera_pose"), pose);
    rmio::json_mat4(params.at("calibration_mat"), K);
    string ply_for_view = params.has("source_scan_ply_path") ? params.at("source_scan_ply_path").str : a.file;
    auto ply_path_for_view = fs::canonical(fs::absolute(fs::path(ply_for_view)));
    auto loaded_ply_path = fs::canonical(fs::absolute(fs::path(a.file)));
    if (ply_path_for_view != loaded_ply_path) {
      cout << "Skipping " << loaded_ply_path << ", rerun with proper ply." << endl;
      p.lock->unlock();
      fs::remove(p.lock_path);
      return;
    }
    // main.cu:202-206 (K column-major: K[8] = cx, K[9] = cy, K[0] = fx)
    float image_width = 2.0f * K[8];
    float image_height = 2.0f * K[9];
    float focal_length_pixels = K[0];
    float fov_radians = 2.0f * atanf(image_width / (2.0f * focal_length_pixels));
    memcpy(p.view.cam2world, pose, sizeof(pose));
    p.view.width = (int32_t)image_width;
    p.view.height = (int32_t)image_height;
    p.view.fov = fov_radians;
    pending.push_back(std::move(p));
  };

  const unsigned hw_threads = std::thread::hardware_concurrency();
  const int view_threads = (int)std::min(hw_threads ? hw_threads : 1u, 16u);
  auto finish = [&](Pending& p, const std::vector<float>& rgbd, double secs) {
    save_outputs(p, rgbd, view_threads);
    cout << fs::canonical(fs::absolute(p.out)) << ": " << (float)secs << " s" << endl;
    p.lock->unlock();
    fs::remove(p.lock_path);
  };

  for (const char* split : {"train", "val"}) {
    const rmio::Json& part = j.at(split);
    for (const auto& kv : part.obj) {
      process(kv.first, kv.second);
      if (!a.batch && !pending.empty()) {
        Pending& p = pending.back();
        std::vector<float> rgbd((size_t)p.view.width * p.view.height * 4);
        rm_frame fr{rgbd.data(), nullptr, nullptr, nullptr};
        auto start = std::chrono::high_resolution_clock::now();
        check(ctx, rm_render(ctx, &p.view, &fr, RM_HOST), "render");
        auto end = std::chrono::high_resolution_clock::now();
        double secs = (float)std::chrono::duration_cast<std::chrono::milliseconds>(end - start).count() / 1000.0f;
        finish(p, rgbd, secs);
        pending.clear();
      }
    }
  }
  if (a.batch && !pending.empty()) {
    std::vector<rm_view> views;
    for (auto& p : pending) views.push_back(p.view);
    if (a.autotune) {
      rm_launch L;
      int32_t leaf;
      float ms;
      check(ctx, rm_autotune(ctx, views.data(), (int32_t)std::min<size_t>(views.size(), 16), &L, &leaf, &ms), "autotune");
    }
    std::vector<std::vector<float>> images(pending.size());
    std::vector<rm_frame> frames(pending.size());
    for (size_t i = 0; i < pending.size(); ++i) {
      images[i].resize((size_t)views[i].width * views[i].height * 4);
      frames[i] = rm_frame{images[i].data(), nullptr, nullptr, nullptr};
    }
    auto start = std::chrono::high_resolution_clock::now();
    check(ctx, rm_render_batch(ctx, views.data(), (int32_t)views.size(), frames.data(), RM_HOST), "batch render");
    auto end = std::chrono::high_resolution_clock::now();
    double per = std::chrono::duration_cast<std::chrono::milliseconds>(end - start).count() / 1000.0 / pending.size();
    // encode and write every view's files on the host cores (PNG deflate
    // dominates the batch's wall time otherwise), then print and release
    // the locks in view order, as one view at a time would
    const size_t nv = pending.size();
    unsigned nt = std::thread::hardware_concurrency();
    nt = (unsigned)std::max<size_t>(1, std::min<size_t>({nt ? nt : 4u, 32u, nv}));
    // A view whose files could not be written keeps its .lock file, as a
    // run of the reference that stops in that view's output would; every
    // view written before or after it is still reported and unlocked, and
    // the first error is raised after that.
    std::vector<std::exception_ptr> err(nv);
    std::vector<std::thread> workers;
    for (unsigned w = 0; w < nt; ++w)
      workers.emplace_back([&, w] {
        for (size_t i = w; i < nv; i += nt) {
          try {
            save_outputs(pending[i], images[i], 1);
          } catch (...) {
            err[i] = std::current_exception();
          }
        }
      });
    for (auto& t : workers) t.join();
    std::exception_ptr first;
    for (size_t i = 0; i < nv; ++i) {
      if (err[i]) {
        if (!first) first = err[i];
        continue;
      }
      cout << fs::canonical(fs::absolute(pending[i].out)) << ": " << (float)per << " s" << endl;
      pending[i].lock->unlock();
      fs::remove(pending[i].lock_path);
    }
    if (first) std::rethrow_exception(first);
  }
  return EXIT_SUCCESS;
}

}  // namespace

int main(int argc, char** argv) {
  Args a;
  try {
    if (!parse_args(argc, argv, a)) return 109;
    if (a.file.empty()) {
      std::cerr << "--file is required" << endl;
      return EXIT_FAILURE;
    }
    return run(a);
  } catch (const std::exception& e) {
    std::cerr << e.what() << endl;
    return EXIT_FAILURE;
  }
}
