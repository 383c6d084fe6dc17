// io.hpp -- file formats of the reference's process boundary, written for
// this project: PLY point clouds (src/pointcloud.cpp:43-58 via happly), the
// .kdtree.radii cache (a Boost text archive of std::vector<float>,
// main.cu:115-127), the view-matrices JSON (README.md:38-98), and the
// colour PNG / depth PNG / depth .npy outputs (src/utils.cu:151-192).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace rmio {

struct Cloud {
  std::vector<float> xyz;    // 3 per point
  std::vector<uint8_t> rgb;  // 3 per point
  size_t size() const { return xyz.size() / 3; }
};

// Reads vertex x, y, z (any numeric type, converted through double to
// float as happly + glm::vec4 do) and red, green, blue (uchar) from an
// ascii or binary (little/big endian) PLY.  Throws std::runtime_error.
Cloud load_ply(const std::string& path);
void save_ply(const std::string& path, const Cloud& c);

// Boost text archive of std::vector<float>.  The reader accepts the
// "22 serialization::archive <version>" header followed by optional class
// tracking/version tokens, the element count, an optional item version and
// the values; the writer emits the layout Boost 1.71 produces with 9
// significant digits, which round-trips float32 exactly.
std::vector<float> read_radii_archive(const std::string& path);
void write_radii_archive(const std::string& path, const std::vector<float>& radii);

// Minimal JSON value (objects keep keys sorted, like nlohmann::json's
// default std::map, so iteration order matches the reference's).
struct Json {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Json> arr;
  std::map<std::string, Json> obj;
  const Json& at(const std::string& key) const;
  bool has(const std::string& key) const { return kind == Object && obj.count(key) > 0; }
};
Json parse_json(const std::string& text);
Json load_json(const std::string& path);

// Row-major JSON 4x4 -> column-major float[16] (glm::from_json, src/utils.cu:137-149).
void json_mat4(const Json& j, float out[16]);

// PNG writers (zlib-compressed, 8-bit).  Rows are written top-down from
// `rows`, which callers pass already flipped.  With threads > 1 an image of
// at least 1 MB is deflated in that many row slices at once (one zlib
// stream: each slice ends on a byte-aligned flush and the slices' Adler-32
// sums are combined), so the decoded pixels are the same.
void write_png(const std::string& path, int width, int height, int channels, const uint8_t* rows,
               int threads = 1);
// float32 (H, W) C-order .npy
void write_npy_f32(const std::string& path, int height, int width, const float* data);

// The reference's encodings of one RGBA32F frame (row 0 = bottom):
//   colour PNG: RGBA8 with alpha forced to 255, (uchar)(v * 255), flipped;
//   depth PNG: 0 where |d - 1| < 1e-5, else (uint8)clamp(2.55 * d, 0, 255), flipped;
//   depth .npy: raw depth, flipped.
void encode_colour_rgba8(int width, int height, const float* rgbd, std::vector<uint8_t>& out);
void encode_depth_u8(int width, int height, const float* rgbd, std::vector<uint8_t>& out,
                     std::vector<float>& depth_flipped);

}  // namespace rmio
