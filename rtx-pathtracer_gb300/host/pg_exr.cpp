// pg_exr.cpp - OpenEXR scanline images, the subset the reference's scenes and
// golden renders use (CommonOps.cpp:12-65 reads and writes them through the
// OpenEXR library, which this build does not have): HALF / FLOAT / UINT
// channels, NONE, ZIPS, ZIP and PIZ compression, increasing or decreasing
// line order.  ZIP blocks are zlib streams; they are inflated here by a
// project-written decoder of the DEFLATE format (RFC 1950 / 1951), then the
// EXR byte predictor and the two-half interleave are undone.  PIZ blocks go
// through the project's restatement of OpenEXR's Huffman, wavelet and value
// table steps (piz_decode).  The writer stores FLOAT channels without
// compression.
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

// ---------------------------------------------------------------------------
// PIZ (OpenEXR's wavelet + Huffman compression of 32-line chunks)
//
// Chunk layout: the bitmap of 16-bit values present (first and last non-zero
// byte, then those bytes), the length of the Huffman stream, the stream.  The
// stream holds the code lengths of symbols [im, iM] (6-bit fields, with runs
// of zero lengths coded as 59..62 for 2..5 zeros and 63 + 8 bits for 6..261
// zeros), codes assigned longest-first in symbol order, then nBits of codes;
// symbol iM repeats the previous value (8-bit count).  The decoded values are,
// per channel, a 2-D Haar-like wavelet transform (14-bit or modular 16-bit
// lifting) of the channel's lines, over indices of the values present.
// ---------------------------------------------------------------------------
struct PizBits {
    const uint8_t *p, *end;
    uint64_t c = 0;
    int lc = 0;
    bool get(int nb, uint32_t &v) {
        while (lc < nb) {
            if (p >= end) return false;
            c = (c << 8) | *p++;
            lc += 8;
        }
        lc -= nb;
        v = (uint32_t)((c >> lc) & ((1ull << nb) - 1));
        return true;
    }
};

bool huf_decode(const uint8_t *d, size_t n, uint16_t *out, size_t nout) {
    constexpr uint32_t kEncSize = 65537;
    if (n == 0) return nout == 0;
    if (n < 20) return false;
    const uint32_t im = rd<uint32_t>(d), iM = rd<uint32_t>(d + 4), nbits = rd<uint32_t>(d + 12);
    if (im >= kEncSize || iM >= kEncSize || im > iM) return false;
    std::vector<uint8_t> len(kEncSize, 0);
    PizBits tb{d + 20, d + n};
    for (uint32_t i = im; i <= iM; ++i) {
        uint32_t l;
        if (!tb.get(6, l)) return false;
        if (l >= 59) {
            uint32_t run;
            if (l == 63) {
                uint32_t z;
                if (!tb.get(8, z)) return false;
                run = z + 6;
            } else {
                run = l - 59 + 2;
            }
            if (i + run > iM + 1) return false;
            i += run - 1;  // lengths stay 0
        } else {
            len[i] = (uint8_t)l;
        }
    }
    // codes: per length, the first code, longest lengths taking the smallest values
    uint64_t cnt[59] = {0}, base[59] = {0};
    for (uint32_t i = 0; i < kEncSize; ++i) cnt[len[i]]++;
    uint64_t c = 0;
    for (int l = 58; l > 0; --l) {
        base[l] = c;
        c = (c + cnt[l]) >> 1;
    }
    std::vector<std::vector<uint32_t>> sym(59);
    for (uint32_t i = 0; i < kEncSize; ++i)
        if (len[i]) sym[len[i]].push_back(i);  // symbol order within a length
    const uint8_t *ds = tb.p;  // the code stream starts at the next whole byte
    if ((uint64_t)(d + n - ds) * 8 < nbits) return false;
    uint64_t pos = 0;
    auto bit = [&]() -> uint32_t {
        const uint32_t b = (ds[pos >> 3] >> (7 - (pos & 7))) & 1u;
        ++pos;
        return b;
    };
    size_t o = 0;
    while (pos < nbits) {
        uint64_t code = 0;
        int l = 0;
        uint32_t s = 0xFFFFFFFFu;
        while (pos < nbits && l < 58) {
            code = (code << 1) | bit();
            ++l;
            if (!sym[l].empty() && code >= base[l] && code < base[l] + sym[l].size()) {
                s = sym[l][code - base[l]];
                break;
            }
        }
        if (s == 0xFFFFFFFFu) return false;
        if (s == iM) {  // run of the previous value
            if (pos + 8 > nbits || o == 0) return false;
            uint32_t r = 0;
            for (int k = 0; k < 8; ++k) r = (r << 1) | bit();
            if (o + r > nout) return false;
            const uint16_t prev = out[o - 1];
            for (uint32_t k = 0; k < r; ++k) out[o++] = prev;
        } else {
            if (o >= nout) return false;
            out[o++] = (uint16_t)s;
        }
    }
    return o == nout;
}

inline void wdec14(uint16_t l, uint16_t h, uint16_t &a, uint16_t &b) {
    const int ls = (int16_t)l, hi = (int16_t)h;
    const int ai = ls + (hi & 1) + (hi >> 1);
    a = (uint16_t)(int16_t)ai;
    b = (uint16_t)(int16_t)(ai - hi);
}
inline void wdec16(uint16_t l, uint16_t h, uint16_t &a, uint16_t &b) {
    const int m = l, dd = h;
    const int bb = (m - (dd >> 1)) & 0xFFFF;
    const int aa = (dd + bb - 0x8000) & 0xFFFF;
    b = (uint16_t)bb;
    a = (uint16_t)aa;
}

// Inverse wavelet of an nx x ny array (element strides ox, oy) whose values
// index at most mx.
void wav2_decode(uint16_t *in, int nx, int ox, int ny, int oy, int mx) {
    const bool w14 = mx < (1 << 14);
    auto dec = [&](uint16_t l, uint16_t h, uint16_t &a, uint16_t &b) {
        if (w14)
            wdec14(l, h, a, b);
        else
            wdec16(l, h, a, b);
    };
    const int n = nx > ny ? ny : nx;
    int p = 1;
    while (p <= n) p <<= 1;
    p >>= 1;
    int p2 = p;
    p >>= 1;
    while (p >= 1) {
        long py = 0;
        const long ey = (long)oy * (ny - p2);
        const long oy1 = (long)oy * p, oy2 = (long)oy * p2, ox1 = (long)ox * p, ox2 = (long)ox * p2;
        uint16_t i00, i01, i10, i11;
        for (; py <= ey; py += oy2) {
            long px = py;
            const long ex = py + (long)ox * (nx - p2);
            for (; px <= ex; px += ox2) {
                const long p01 = px + ox1, p10 = px + oy1, p11 = p10 + ox1;
                dec(in[px], in[p10], i00, i10);
                dec(in[p01], in[p11], i01, i11);
                dec(i00, i01, in[px], in[p01]);
                dec(i10, i11, in[p10], in[p11]);
            }
            if (nx & p) {
                const long p10 = px + oy1;
                dec(in[px], in[p10], i00, in[p10]);
                in[px] = i00;
            }
        }
        if (ny & p) {
            long px = py;
            const long ex = py + (long)ox * (nx - p2);
            for (; px <= ex; px += ox2) {
                const long p01 = px + ox1;
                dec(in[px], in[p01], i00, in[p01]);
                in[px] = i00;
            }
        }
        p2 = p;
        p >>= 1;
    }
}

// One PIZ chunk of nl lines of width W into the uncompressed line layout
// (per line, each channel's W samples), `want` bytes.
bool piz_decode(const uint8_t *src, size_t n, const std::vector<Channel> &chans, int W, int nl, size_t want,
                std::vector<uint8_t> &out) {
    if (n < 4) return false;
    const uint16_t mn = rd<uint16_t>(src), mxz = rd<uint16_t>(src + 2);
    size_t p = 4;
    std::vector<uint8_t> bitmap(8192, 0);
    if (mxz >= 8192) return false;
    if (mn <= mxz) {
        const size_t k = (size_t)mxz - mn + 1;
        if (p + k > n) return false;
        memcpy(&bitmap[mn], src + p, k);
        p += k;
    }
    std::vector<uint16_t> lut(65536, 0);
    int k = 0;
    for (int i = 0; i < 65536; ++i)
        if (i == 0 || (bitmap[i >> 3] & (1 << (i & 7)))) lut[k++] = (uint16_t)i;
    const int max_value = k - 1;
    if (p + 4 > n) return false;
    const int32_t len = rd<int32_t>(src + p);
    p += 4;
    if (len < 0 || p + (size_t)len > n || want % 2) return false;
    std::vector<uint16_t> buf(want / 2);
    if (!huf_decode(src + p, (size_t)len, buf.data(), buf.size())) return false;
    std::vector<size_t> start;
    size_t at = 0;
    for (auto &c : chans) {
        const int size = pixel_bytes(c.type) / 2;
        start.push_back(at);
        for (int j = 0; j < size; ++j) wav2_decode(&buf[at + j], W, size, nl, W * size, max_value);
        at += (size_t)W * nl * size;
    }
    if (at != buf.size()) return false;
    for (auto &v : buf) v = lut[v];
    out.resize(want);
    size_t o = 0;
    for (int l = 0; l < nl; ++l)
        for (size_t c = 0; c < chans.size(); ++c) {
            const size_t cnt = (size_t)W * (pixel_bytes(chans[c].type) / 2);
            for (size_t i = 0; i < cnt; ++i) {
                const uint16_t v = buf[start[c] + (size_t)l * cnt + i];
                out[o++] = (uint8_t)(v & 0xFF);
                out[o++] = (uint8_t)(v >> 8);
            }
        }
    return true;
}

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
    else if (compression == 4) lines = 32;                      // PIZ
    else {
        err = path + ": compression " + std::to_string(compression) + " is not supported (NONE, ZIPS, ZIP, PIZ are)";
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
        } else if (compression == 4) {
            if (!piz_decode(src, (size_t)size, chans, W, nl, want, raw)) {
                err = path + ": cannot decode PIZ chunk " + std::to_string(c);
                return false;
            }
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
