// pg_png.cpp - PNG decoding (ISO/IEC 15948): chunk walk, the IDAT stream
// through the project's zlib inflate, the five scanline filters, and the
// expansion of each colour type to RGBA8.  The reference loads its textures
// with stb_image as 4-channel images (src/SceneLoader.cpp:184-233); grey
// expands to RGB, missing alpha is 255, palette entries take their tRNS alpha.
#include "pg_png.h"

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>

#include "pg_exr.h"

namespace pg {
namespace {

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

}  // namespace

bool decode_png(const uint8_t *d, size_t n, uint32_t &width, uint32_t &height, std::vector<uint8_t> &rgba,
                std::string &err) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (n < 8 || memcmp(d, sig, 8) != 0) {
        err = "not a PNG file";
        return false;
    }
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    size_t pos = 8;
    bool have_header = false, end = false;
    while (!end) {
        if (pos + 12 > n) {
            err = "truncated PNG chunk";
            return false;
        }
        const uint32_t len = be32(d + pos);
        const uint8_t *type = d + pos + 4, *body = d + pos + 8;
        if (len > n - pos - 12) {
            err = "truncated PNG chunk";
            return false;
        }
        if (!memcmp(type, "IHDR", 4)) {
            if (len < 13) {
                err = "short IHDR";
                return false;
            }
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            have_header = true;
        } else if (!memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!memcmp(type, "IEND", 4)) {
            end = true;
        }
        pos += 12 + (size_t)len;
    }
    if (!have_header || w == 0 || h == 0 || w > (1u << 15) || h > (1u << 15)) {
        err = "bad PNG header";
        return false;
    }
    if (depth != 8 || interlace != 0) {
        err = "only 8-bit, non-interlaced PNG images are decoded";
        return false;
    }
    int channels;
    switch (ctype) {
        case 0: channels = 1; break;
        case 2: channels = 3; break;
        case 3: channels = 1; break;
        case 4: channels = 2; break;
        case 6: channels = 4; break;
        default: err = "unknown PNG colour type"; return false;
    }
    if (ctype == 3 && (plte.empty() || plte.size() % 3 != 0)) {
        err = "palette image without PLTE";
        return false;
    }
    std::vector<uint8_t> raw;
    if (!zlib_inflate(idat.data(), idat.size(), raw)) {
        err = "cannot inflate PNG image data";
        return false;
    }
    const size_t stride = (size_t)w * channels;
    if (raw.size() < (stride + 1) * h) {
        err = "PNG image data too short";
        return false;
    }
    // undo the scanline filters in place (bytes per pixel = channels at 8 bits)
    std::vector<uint8_t> px(stride * h);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t f = raw[y * (stride + 1)];
        const uint8_t *src = &raw[y * (stride + 1) + 1];
        uint8_t *row = &px[y * stride];
        const uint8_t *up = y ? &px[(y - 1) * stride] : nullptr;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= (size_t)channels ? row[i - channels] : 0;
            const int b = up ? up[i] : 0;
            const int c = (up && i >= (size_t)channels) ? up[i - channels] : 0;
            int v = src[i];
            switch (f) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: err = "unknown PNG filter"; return false;
            }
            row[i] = (uint8_t)v;
        }
    }
    rgba.assign((size_t)w * h * 4, 255);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        uint8_t *o = &rgba[4 * i];
        const uint8_t *p = &px[i * channels];
        switch (ctype) {
            case 0: o[0] = o[1] = o[2] = p[0]; break;
            case 2: o[0] = p[0], o[1] = p[1], o[2] = p[2]; break;
            case 3: {
                const size_t e = p[0];
                if (3 * e + 2 >= plte.size()) {
                    err = "PNG palette index out of range";
                    return false;
                }
                o[0] = plte[3 * e], o[1] = plte[3 * e + 1], o[2] = plte[3 * e + 2];
                if (e < trns.size()) o[3] = trns[e];
                break;
            }
            case 4: o[0] = o[1] = o[2] = p[0], o[3] = p[1]; break;
            default: memcpy(o, p, 4); break;
        }
    }
    width = w;
    height = h;
    return true;
}

bool read_png(const std::string &path, uint32_t &width, uint32_t &height, std::vector<uint8_t> &rgba,
              std::string &err) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        err = "cannot open " + path;
        return false;
    }
    const std::vector<uint8_t> data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (!decode_png(data.data(), data.size(), width, height, rgba, err)) {
        err = path + ": " + err;
        return false;
    }
    return true;
}

}  // namespace pg
