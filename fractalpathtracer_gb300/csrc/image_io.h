// image_io.h -- PNG and Radiance RGBE I/O and the reference's image metrics (host code).
#pragma once

#include <stdint.h>
#include <stddef.h>
#include <string>
#include <vector>

namespace fpt {

struct Image {
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> rgba;  // row 0 = top
};

// Writes an 8-bit RGBA PNG (zlib stream of stored deflate blocks).
bool write_png(const char *path, uint32_t w, uint32_t h, const uint8_t *rgba, std::string &err);
// Reads an 8-bit RGB/RGBA/grey PNG (any deflate stream, non-interlaced).
bool read_png(const char *path, Image &out, std::string &err);

struct HdrImage {
    uint32_t width = 0, height = 0;
    std::vector<float> rgb;
};
// Radiance RLE reader (src/metal_bridge.mm:2184-2259).
bool read_radiance_hdr(const char *path, HdrImage &out, std::string &err);
// float -> half conversion used by the reference's HDRI LUT (src/metal_bridge.mm:2163-2176).
uint16_t reference_float_to_half(float value);

// Image metrics (src/metal_bridge.mm:2383-2495, 6078-6104).
struct ImageMetrics {
    double mae, rmse, max_abs, changed_pct, ssim, lf_ssim;
    size_t unique_baseline, unique_candidate;
};
ImageMetrics compare_rgba(const uint8_t *a, const uint8_t *b, uint32_t w, uint32_t h);
size_t unique_colour_sample(const uint8_t *rgba, size_t pixels);

}  // namespace fpt
