// rmio_c.cpp -- C entry points over io.hpp (librm_io.so), so the file
// formats of the reference's process boundary can be used and tested
// without a GPU.  Every function returns 0 on success, -1 on failure with
// the message available from rmio_last_error() (per thread).
#include <algorithm>
#include <cstring>
#include <string>
#include <thread>

#include "io.hpp"
#include "rmio.h"

namespace {
thread_local std::string g_err;
thread_local rmio::Cloud g_cloud;
thread_local std::vector<float> g_radii;

template <class F>
int guarded(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
}  // namespace

extern "C" {

const char* rmio_last_error(void) { return g_err.c_str(); }

int rmio_ply_open(const char* path, int64_t* n_out) {
  return guarded([&] {
    g_cloud = rmio::load_ply(path);
    *n_out = (int64_t)g_cloud.size();
  });
}

int rmio_ply_take(float* xyz, uint8_t* rgb) {
  return guarded([&] {
    memcpy(xyz, g_cloud.xyz.data(), g_cloud.xyz.size() * sizeof(float));
    if (rgb) memcpy(rgb, g_cloud.rgb.data(), g_cloud.rgb.size());
    g_cloud = rmio::Cloud();
  });
}

int rmio_ply_save(const char* path, const float* xyz, const uint8_t* rgb, int64_t n) {
  return guarded([&] {
    rmio::Cloud c;
    c.xyz.assign(xyz, xyz + 3 * n);
    c.rgb.assign(rgb, rgb + 3 * n);
    rmio::save_ply(path, c);
  });
}

int rmio_radii_open(const char* path, int64_t* n_out) {
  return guarded([&] {
    g_radii = rmio::read_radii_archive(path);
    *n_out = (int64_t)g_radii.size();
  });
}

int rmio_radii_take(float* out) {
  return guarded([&] {
    memcpy(out, g_radii.data(), g_radii.size() * sizeof(float));
    g_radii.clear();
  });
}

int rmio_radii_save(const char* path, const float* radii, int64_t n) {
  return guarded([&] { rmio::write_radii_archive(path, std::vector<float>(radii, radii + n)); });
}

int rmio_write_frame(const char* colour_png, const char* depth_png, int32_t width, int32_t height,
                     const float* rgbd) {
  return guarded([&] {
    std::vector<uint8_t> png, dpng;
    std::vector<float> depth;
    const unsigned hw = std::thread::hardware_concurrency();
    const int threads = (int)std::min(hw ? hw : 1u, 16u);  // one frame: its PNGs deflate in row slices
    rmio::encode_colour_rgba8(width, height, rgbd, png);
    rmio::write_png(colour_png, width, height, 4, png.data(), threads);
    rmio::encode_depth_u8(width, height, rgbd, dpng, depth);
    rmio::write_npy_f32(std::string(depth_png) + ".npy", height, width, depth.data());
    rmio::write_png(depth_png, width, height, 1, dpng.data(), threads);
  });
}

int rmio_json_mat4(const char* json_text, float* out16) {
  return guarded([&] { rmio::json_mat4(rmio::parse_json(json_text), out16); });
}

}  // extern "C"
