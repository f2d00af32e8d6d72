// pg_png.h - PNG images for material textures: 8-bit grey, grey + alpha, RGB,
// RGBA and palette images (non-interlaced), decoded to RGBA8 rows from the top.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pg {

bool read_png(const std::string &path, uint32_t &width, uint32_t &height, std::vector<uint8_t> &rgba,
              std::string &err);
bool decode_png(const uint8_t *data, size_t n, uint32_t &width, uint32_t &height, std::vector<uint8_t> &rgba,
                std::string &err);

}  // namespace pg
