// pg_jpeg.h - baseline (sequential, Huffman-coded, 8-bit) JPEG images for
// material textures, decoded to RGBA8 rows from the top (alpha 255).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pg {

bool decode_jpeg(const uint8_t *data, size_t n, uint32_t &width, uint32_t &height, std::vector<uint8_t> &rgba,
                 std::string &err);

}  // namespace pg
