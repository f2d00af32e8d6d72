// pg_exr.cpp - OpenEXR scanline images, the subset the reference's scenes and
// golden renders use (CommonOps.cpp:12-65 reads and writes them through the
// OpenEXR library, which this build does not have): HALF / FLOAT / UINT
// channels, NONE, ZIPS and ZIP compression, increasing or decreasing line
// order.  ZIP blocks are zlib streams; they are inflated here by a
// project-written decoder of the DEFLATE format (RFC 1950 / 1951), then the
// EXR byte predictor and the two-half interleave are undone.  The writer
// stores FLOAT channels without compression.
#include "pg_exr.h"

#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

namespace pg {
namespace {

// ---------------------------------------------------------------------------
// DEFLATE (RFC 1951)
// ---------------------------------------------------------------------------

struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    bool fail = false;
    int bit() {
        if (bitcnt == 0) {
            if (pos >= n) {
                fail = true;
                return 0;
            }
            bitbuf = p[pos++];
            bitcnt = 8;
        }
        const int b = (int)(bitbuf & 1u);
        bitbuf >>= 1;
        --bitcnt;
        return b;
    }
    uint32_t bits(int k) {  // least significant bit first
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
    void align() { bitcnt = 0; }
};

// Canonical Huffman code: symbol counts per length and symbols in code order.
struct Huffman {
    uint16_t count[16] = {0};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t *lengths, int n) {
        memset(count, 0, sizeof count);
        for (int i = 0; i < n; ++i) ++count[lengths[i]];
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; ++len) {
            left <<= 1;
            left -= count[len];
            if (left < 0) return false;  // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; ++len) offs[len + 1] = (uint16_t)(offs[len] + count[len]);
        symbol.assign(n, 0);
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(BitReader &br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= br.bit();
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
            if (br.fail) return -1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99,
                               115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
                                1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11,
                                12, 12, 13, 13};

bool inflate_codes(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out) {
    for (;;) {
        const int sym = lit.decode(br);
        if (sym < 0) return false;
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            const int li = sym - 257;
            if (li >= 29) return false;
            const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int ds = dist.decode(br);
            if (ds < 0 || ds >= 30) return false;
            const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (d > out.size() || br.fail) return false;
            const size_t from = out.size() - d;
            for (size_t i = 0; i < len; ++i) out.push_back(out[from + i]);
        }
    }
}

bool inflate_raw(const uint8_t *src, size_t n, std::vector<uint8_t> &out) {
    BitReader br{src, n};
    int last;
    do {
        last = br.bit();
        const uint32_t type = br.bits(2);
        if (br.fail) return false;
        if (type == 0) {  // stored
            br.align();
            if (br.pos + 4 > n) return false;
            const uint16_t len = (uint16_t)(src[br.pos] | (src[br.pos + 1] << 8));
            const uint16_t nlen = (uint16_t)(src[br.pos + 2] | (src[br.pos + 3] << 8));
            br.pos += 4;
            if ((uint16_t)~nlen != len || br.pos + len > n) return false;
            out.insert(out.end(), src + br.pos, src + br.pos + len);
            br.pos += len;
        } else if (type == 1) {  // fixed codes
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            for (int i = 0; i < 30; ++i) d[i] = 5;
            Huffman lit, dist;
            if (!lit.build(l, 288) || !dist.build(d, 30) || !inflate_codes(br, lit, dist, out)) return false;
        } else if (type == 2) {  // dynamic codes
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) return false;
            uint8_t lens[320] = {0};
            int i = 0;
            while (i < hlit + hdist) {
                const int sym = clh.decode(br);
                if (sym < 0) return false;
                if (sym < 16) {
                    lens[i++] = (uint8_t)sym;
                } else {
                    int rep = 0;
                    uint8_t v = 0;
                    if (sym == 16) {
                        if (i == 0) return false;
                        v = lens[i - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (i + rep > hlit + hdist) return false;
                    while (rep--) lens[i++] = v;
                }
            }
            Huffman lit, dist;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist) || !inflate_codes(br, lit, dist, out))
                return false;
        } else {
            return false;
        }
    } while (!last);
    return !br.fail;
}

// zlib stream (RFC 1950): 2-byte header, DEFLATE data, Adler-32 (checked)
bool inflate_zlib(const uint8_t *src, size_t n, std::vector<uint8_t> &out) {
    if (n < 6 || (src[0] & 0x0F) != 8 || ((src[0] << 8) | src[1]) % 31 != 0 || (src[1] & 0x20)) return false;
    if (!inflate_raw(src + 2, n - 6, out)) return false;
    uint32_t a = 1, b = 0;
    for (uint8_t c : out) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    const uint8_t *t = src + n - 4;
    const uint32_t want = ((uint32_t)t[0] << 24) | ((uint32_t)t[1] << 16) | ((uint32_t)t[2] << 8) | t[3];
    return ((b << 16) | a) == want;
}

// ---------------------------------------------------------------------------
// EXR
// ---------------------------------------------------------------------------

float half_to_float(uint16_t h) {
    const uint32_t s = (uint32_t)(h >> 15), e = (uint32_t)(h >> 10) & 0x1Fu, m = h & 0x3FFu;
    float v;
    if (e == 0) v = std::ldexp((float)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((float)(m | 0x400u), (int)e - 25);
    return s ? -v : v;
}

template <class T>
T rd(const uint8_t *p) {
    T v;
    memcpy(&v, p, sizeof v);  // EXR is little-endian, as both build hosts are
    return v;
}

struct Channel {
    std::string name;
    int32_t type;  // 0 UINT, 1 HALF, 2 FLOAT
    int32_t xs, ys;
};

int pixel_bytes(int32_t type) { return type == 1 ? 2 : 4; }

}  // namespace

bool read_exr(const std::string &path, ExrImage &img, std::string &err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<uint8_t> d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    const size_t n = d.size();
    if (n < 8 || rd<int32_t>(&d[0]) != 20000630) {
        err = path + ": not an OpenEXR file";
        return false;
    }
    const uint32_t flags = rd<uint32_t>(&d[4]);
    if ((flags & 0xFFu) != 2 || (flags & 0x200u) || (flags & 0x1000u)) {
        err = path + ": only single-part scanline EXR version 2 is read";
        return false;
    }
    size_t pos = 8;
    std::vector<Channel> chans;
    int compression = -1, line_order = 0;
    int32_t dw[4] = {0, 0, -1, -1};
    auto cstr = [&](std::string &out) {
        const size_t s = pos;
        while (pos < n && d[pos]) ++pos;
        if (pos >= n) return false;
        out.assign((const char *)&d[s], pos - s);
        ++pos;
        return true;
    };
    for (;;) {
        std::string name, type;
        if (!cstr(name)) break;
        if (name.empty()) break;
        if (!cstr(type) || pos + 4 > n) {
            err = path + ": truncated header";
            return false;
        }
        const int32_t size = rd<int32_t>(&d[pos]);
        pos += 4;
        if (size < 0 || pos + (size_t)size > n) {
            err = path + ": truncated header";
            return false;
        }
        const uint8_t *v = &d[pos];
        if (name == "channels" && type == "chlist") {
            size_t q = 0;
            while (q < (size_t)size && v[q]) {
                Channel c;
                const size_t s0 = q;
                while (q < (size_t)size && v[q]) ++q;
                c.name.assign((const char *)v + s0, q - s0);
                ++q;
                if (q + 16 > (size_t)size) break;
                c.type = rd<int32_t>(v + q);
                c.xs = rd<int32_t>(v + q + 8);
                c.ys = rd<int32_t>(v + q + 12);
                q += 16;
                chans.push_back(c);
            }
        } else if (name == "compression") {
            compression = v[0];
        } else if (name == "dataWindow" && size == 16) {
            for (int i = 0; i < 4; ++i) dw[i] = rd<int32_t>(v + 4 * i);
        } else if (name == "lineOrder") {
            line_order = v[0];
        }
        pos += (size_t)size;
    }
    const int32_t W = dw[2] - dw[0] + 1, H = dw[3] - dw[1] + 1;
    if (W <= 0 || H <= 0 || chans.empty()) {
        err = path + ": empty image or no channels";
        return false;
    }
    for (auto &c : chans)
        if (c.xs != 1 || c.ys != 1 || c.type < 0 || c.type > 2) {
            err = path + ": subsampled or unknown channel " + c.name;
            return false;
        }
    int lines;
    if (compression == 0 || compression == 2) lines = 1;       // NONE, ZIPS
    else if (compression == 3) lines = 16;                      // ZIP
    else {
        err = path + ": compression " + std::to_string(compression) + " is not supported (NONE, ZIPS, ZIP are)";
        return false;
    }
    (void)line_order;  // chunks carry their own y
    size_t row_bytes = 0;
    for (auto &c : chans) row_bytes += (size_t)W * pixel_bytes(c.type);
    const int chunks = (H + lines - 1) / lines;
    if (pos + 8 * (size_t)chunks > n) {
        err = path + ": truncated offset table";
        return false;
    }
    int cr = -1, cg = -1, cb = -1, cy = -1;
    for (size_t i = 0; i < chans.size(); ++i) {
        if (chans[i].name == "R") cr = (int)i;
        if (chans[i].name == "G") cg = (int)i;
        if (chans[i].name == "B") cb = (int)i;
        if (chans[i].name == "Y") cy = (int)i;
    }
    if (!((cr >= 0 && cg >= 0 && cb >= 0) || cy >= 0)) {
        err = path + ": no R, G, B (or Y) channels";
        return false;
    }
    img.width = (uint32_t)W;
    img.height = (uint32_t)H;
    img.rgb.assign((size_t)W * H * 3, 0.0f);
    std::vector<uint8_t> raw, tmp;
    for (int c = 0; c < chunks; ++c) {
        const uint64_t off = rd<uint64_t>(&d[pos + 8 * (size_t)c]);
        if (off + 8 > n) {
            err = path + ": bad chunk offset";
            return false;
        }
        const int32_t y0 = rd<int32_t>(&d[off]) - dw[1];
        const int32_t size = rd<int32_t>(&d[off + 4]);
        if (size < 0 || off + 8 + (uint64_t)size > n || y0 < 0 || y0 >= H) {
            err = path + ": bad chunk";
            return false;
        }
        const int nl = std::min(lines, H - y0);
        const size_t want = row_bytes * (size_t)nl;
        const uint8_t *src = &d[off + 8];
        if ((size_t)size == want) {  // stored uncompressed (also allowed for ZIP chunks)
            raw.assign(src, src + want);
        } else {
            tmp.clear();
            if (compression == 0 || !inflate_zlib(src, (size_t)size, tmp) || tmp.size() != want) {
                err = path + ": cannot inflate chunk " + std::to_string(c);
                return false;
            }
            for (size_t i = 1; i < tmp.size(); ++i) tmp[i] = (uint8_t)(tmp[i - 1] + tmp[i] - 128);  // predictor
            raw.resize(want);
            const size_t half = (want + 1) / 2;
            for (size_t i = 0; i < want; ++i) raw[i] = (i & 1) ? tmp[half + i / 2] : tmp[i / 2];  // interleave
        }
        // per line: each channel's W samples in turn
        for (int l = 0; l < nl; ++l) {
            const uint8_t *line = raw.data() + row_bytes * (size_t)l;
            size_t at = 0;
            for (size_t ci = 0; ci < chans.size(); ++ci) {
                const int pb = pixel_bytes(chans[ci].type);
                int dst = -1;
                if ((int)ci == cr) dst = 0;
                if ((int)ci == cg) dst = 1;
                if ((int)ci == cb) dst = 2;
                for (int x = 0; x < W; ++x) {
                    const uint8_t *q = line + at + (size_t)x * pb;
                    float v;
                    if (chans[ci].type == 1) v = half_to_float(rd<uint16_t>(q));
                    else if (chans[ci].type == 2) v = rd<float>(q);
                    else v = (float)rd<uint32_t>(q);
                    float *px = &img.rgb[3 * ((size_t)(y0 + l) * W + x)];
                    if (dst >= 0) px[dst] = v;
                    else if ((int)ci == cy && cr < 0) px[0] = px[1] = px[2] = v;
                }
                at += (size_t)W * pb;
            }
        }
    }
    return true;
}

bool write_exr(const std::string &path, const float *rgb, uint32_t width, uint32_t height, std::string &err) {
    std::vector<uint8_t> h;
    auto put = [&](const void *p, size_t k) { h.insert(h.end(), (const uint8_t *)p, (const uint8_t *)p + k); };
    auto put_i32 = [&](int32_t v) { put(&v, 4); };
    auto put_str = [&](const char *s) { put(s, strlen(s) + 1); };
    auto attr = [&](const char *name, const char *type, int32_t size) {
        put_str(name);
        put_str(type);
        put_i32(size);
    };
    put_i32(20000630);
    put_i32(2);
    // channels B, G, R (alphabetical), FLOAT
    attr("channels", "chlist", 3 * (2 + 16) + 1);
    for (const char *c : {"B", "G", "R"}) {
        put_str(c);
        put_i32(2);
        const uint8_t plin[4] = {0, 0, 0, 0};
        put(plin, 4);
        put_i32(1);
        put_i32(1);
    }
    h.push_back(0);
    attr("compression", "compression", 1);
    h.push_back(0);
    const int32_t win[4] = {0, 0, (int32_t)width - 1, (int32_t)height - 1};
    attr("dataWindow", "box2i", 16);
    put(win, 16);
    attr("displayWindow", "box2i", 16);
    put(win, 16);
    attr("lineOrder", "lineOrder", 1);
    h.push_back(0);
    const float one = 1.0f, zero2[2] = {0.0f, 0.0f};
    attr("pixelAspectRatio", "float", 4);
    put(&one, 4);
    attr("screenWindowCenter", "v2f", 8);
    put(zero2, 8);
    attr("screenWindowWidth", "float", 4);
    put(&one, 4);
    h.push_back(0);
    const size_t row = (size_t)width * 12;
    uint64_t off = h.size() + 8 * (uint64_t)height;
    for (uint32_t y = 0; y < height; ++y) {
        put(&off, 8);
        off += 8 + row;
    }
    for (uint32_t y = 0; y < height; ++y) {
        put_i32((int32_t)y);
        put_i32((int32_t)row);
        for (int c : {2, 1, 0})
            for (uint32_t x = 0; x < width; ++x) put(&rgb[3 * ((size_t)y * width + x) + c], 4);
    }
    std::ofstream f(path, std::ios::binary);
    if (!f || !f.write((const char *)h.data(), (std::streamsize)h.size())) {
        err = "cannot write " + path;
        return false;
    }
    return true;
}

bool zlib_inflate(const uint8_t *src, size_t n, std::vector<uint8_t> &out) { return inflate_zlib(src, n, out); }

}  // namespace pg
