// pg_exr.h - OpenEXR scanline images (read: NONE / ZIPS / ZIP, HALF / FLOAT /
// UINT; write: FLOAT, no compression), RGB floats row-major from the top row.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pg {

struct ExrImage {
    uint32_t width = 0, height = 0;
    std::vector<float> rgb;
};

bool read_exr(const std::string &path, ExrImage &img, std::string &err);
bool write_exr(const std::string &path, const float *rgb, uint32_t width, uint32_t height, std::string &err);

}  // namespace pg
