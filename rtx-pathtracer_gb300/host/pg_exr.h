// pg_exr.h - OpenEXR scanline images (read: NONE / ZIPS / ZIP / PIZ, HALF / FLOAT /
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
// Decodes a zlib stream (RFC 1950: header, DEFLATE blocks of RFC 1951,
// Adler-32 checked) into out, which must start empty.
bool zlib_inflate(const uint8_t *src, size_t n, std::vector<uint8_t> &out);
bool write_exr(const std::string &path, const float *rgb, uint32_t width, uint32_t height, std::string &err);

}  // namespace pg
