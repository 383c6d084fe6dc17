/*
 * rmio.h -- C ABI of the host-side file formats (librm_io.so, no CUDA):
 * the reference's PLY input (src/pointcloud.cpp:43-58), its .kdtree.radii
 * cache (Boost text archive of std::vector<float>, main.cu:115-127), the
 * row-major JSON matrices (src/utils.cu:137-149) and the per-view outputs
 * (colour PNG, 8-bit depth PNG, float32 depth .npy; src/utils.cu:151-192).
 * Functions return 0 on success, -1 on failure (rmio_last_error()).
 * The *_open / *_take pairs read a file into a per-thread buffer and copy it
 * out once the caller knows the size.
 */
#ifndef RMIO_H
#define RMIO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

const char* rmio_last_error(void);
int rmio_ply_open(const char* path, int64_t* n_out);
int rmio_ply_take(float* xyz, uint8_t* rgb);
int rmio_ply_save(const char* path, const float* xyz, const uint8_t* rgb, int64_t n);
int rmio_radii_open(const char* path, int64_t* n_out);
int rmio_radii_take(float* out);
int rmio_radii_save(const char* path, const float* radii, int64_t n);
/* rgbd: W*H float4 with row 0 at the bottom (the render output layout). */
int rmio_write_frame(const char* colour_png, const char* depth_png, int32_t width, int32_t height,
                     const float* rgbd);
int rmio_json_mat4(const char* json_text, float* out16);

#ifdef __cplusplus
}
#endif
#endif
