// pg_jpeg.cpp - baseline JPEG decoding (ITU-T T.81): the marker segments
// (DQT, SOF0/SOF1, DHT, DRI, SOS), Huffman decoding of the DC differences and
// the AC run/size symbols (T.81 F.2.2), dequantisation in zig-zag order, a
// separable floating-point 8 x 8 inverse DCT (A.3.3), MCU assembly with
// chroma replication for subsampled components, and the JFIF YCbCr -> RGB
// transform.  Progressive and arithmetic-coded images are reported, not
// decoded.  The reference reads its textures with stb_image as 4-channel
// images (src/SceneLoader.cpp:184-233); grey images expand to RGB.
#include "pg_jpeg.h"

#include <math.h>

#include <algorithm>
#include <cstring>

namespace pg {
namespace {

constexpr int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// Canonical Huffman table (T.81 C and F.2.2.3): per code length the largest
// code, the index of its first symbol and the first code.
struct Huff {
    int maxcode[18], valptr[17], mincode[17];
    uint8_t vals[256];
    bool set = false;
    bool build(const uint8_t counts[16], const uint8_t *symbols, int n) {
        if (n > 256) return false;
        memcpy(vals, symbols, (size_t)n);
        int code = 0, k = 0;
        for (int l = 1; l <= 16; ++l) {
            valptr[l] = k;
            mincode[l] = code;
            code += counts[l - 1];
            k += counts[l - 1];
            maxcode[l] = counts[l - 1] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7FFFFFFF;
        set = true;
        return true;
    }
};

struct Bits {
    const uint8_t *d;
    size_t n, pos;
    uint32_t acc = 0;
    int cnt = 0;
    bool marker = false;  // a marker ends the entropy-coded segment: zeros follow
    int bit() {
        if (cnt == 0) {
            uint8_t b = 0;
            if (!marker && pos < n) {
                b = d[pos];
                if (b == 0xFF) {
                    const uint8_t nx = pos + 1 < n ? d[pos + 1] : 0;
                    if (nx == 0x00) {
                        pos += 2;  // stuffed byte
                    } else {
                        marker = true;
                        b = 0;
                    }
                } else {
                    ++pos;
                }
            }
            acc = b;
            cnt = 8;
        }
        --cnt;
        return (acc >> cnt) & 1;
    }
    int bits(int s) {
        int v = 0;
        for (int i = 0; i < s; ++i) v = (v << 1) | bit();
        return v;
    }
    // skip to the next RSTn marker at a restart interval boundary
    void restart() {
        cnt = 0;
        marker = false;
        while (pos + 1 < n && !(d[pos] == 0xFF && d[pos + 1] >= 0xD0 && d[pos + 1] <= 0xD7)) ++pos;
        if (pos + 1 < n) pos += 2;
    }
};

int decode_sym(Bits &b, const Huff &h) {
    int code = b.bit();
    for (int l = 1; l <= 16; ++l) {
        if (h.maxcode[l] >= 0 && code <= h.maxcode[l]) return h.vals[h.valptr[l] + code - h.mincode[l]];
        code = (code << 1) | b.bit();
    }
    return -1;  // corrupt data
}

int extend(int v, int s) { return s == 0 ? 0 : (v < (1 << (s - 1)) ? v - (1 << s) + 1 : v); }

// 8 x 8 inverse DCT of natural-order coefficients into samples (level shift, clamp).
void idct8x8(const float in[64], uint8_t *out, int stride) {
    static float c[8][8];  // c[x][u] = C(u) / 2 cos((2x + 1) u pi / 16)
    static bool init = false;
    if (!init) {
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                c[x][u] = (float)((u == 0 ? sqrt(0.5) : 1.0) * 0.5 * cos((2 * x + 1) * u * M_PI / 16.0));
        init = true;
    }
    float tmp[64];
    for (int v = 0; v < 8; ++v)  // rows: along u
        for (int x = 0; x < 8; ++x) {
            float s = 0.0f;
            for (int u = 0; u < 8; ++u) s += c[x][u] * in[v * 8 + u];
            tmp[v * 8 + x] = s;
        }
    for (int x = 0; x < 8; ++x)
        for (int y = 0; y < 8; ++y) {
            float s = 0.0f;
            for (int v = 0; v < 8; ++v) s += c[y][v] * tmp[v * 8 + x];
            const float p = roundf(s + 128.0f);
            out[y * stride + x] = (uint8_t)(p < 0.0f ? 0.0f : (p > 255.0f ? 255.0f : p));
        }
}

struct Comp {
    int id, h, v, tq, td = 0, ta = 0, pred = 0;
    int bw, bh;                 // blocks across and down (padded to whole MCUs)
    std::vector<uint8_t> plane;  // bw*8 x bh*8 samples
};

uint16_t be16(const uint8_t *p) { return (uint16_t)((p[0] << 8) | p[1]); }

}  // namespace

bool decode_jpeg(const uint8_t *d, size_t n, uint32_t &width, uint32_t &height, std::vector<uint8_t> &rgba,
                 std::string &err) {
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) {
        err = "not a JPEG file";
        return false;
    }
    uint16_t q[4][64] = {};
    Huff dc[4], ac[4];
    std::vector<Comp> comps;
    int W = 0, H = 0, hmax = 1, vmax = 1, restart = 0;
    bool frame = false, done = false;
    size_t pos = 2;
    while (!done) {
        while (pos < n && d[pos] != 0xFF) ++pos;  // tolerate fill bytes
        while (pos < n && d[pos] == 0xFF) ++pos;
        if (pos >= n) {
            err = "JPEG ends before the image data";
            return false;
        }
        const uint8_t m = d[pos++];
        if (m == 0xD8 || (m >= 0xD0 && m <= 0xD7)) continue;
        if (m == 0xD9) break;
        if (pos + 2 > n) {
            err = "truncated JPEG segment";
            return false;
        }
        const size_t len = be16(d + pos);
        if (len < 2 || pos + len > n) {
            err = "truncated JPEG segment";
            return false;
        }
        const uint8_t *s = d + pos + 2;
        const size_t sl = len - 2;
        switch (m) {
            case 0xDB: {  // DQT
                size_t i = 0;
                while (i < sl) {
                    const int pq = s[i] >> 4, tq = s[i] & 3;
                    ++i;
                    if (i + (pq ? 128 : 64) > sl) {
                        err = "bad DQT";
                        return false;
                    }
                    for (int k = 0; k < 64; ++k) q[tq][k] = pq ? be16(s + i + 2 * k) : s[i + k];
                    i += pq ? 128 : 64;
                }
                break;
            }
            case 0xC0:
            case 0xC1: {  // baseline / extended sequential, Huffman
                if (sl < 6 || s[0] != 8) {
                    err = "only 8-bit sequential JPEG images are decoded";
                    return false;
                }
                H = be16(s + 1);
                W = be16(s + 3);
                const int nc = s[5];
                if (W <= 0 || H <= 0 || W > 32768 || H > 32768 || (nc != 1 && nc != 3) || sl < 6 + 3 * (size_t)nc) {
                    err = "unsupported JPEG frame (grey or YCbCr only)";
                    return false;
                }
                comps.resize((size_t)nc);
                for (int c = 0; c < nc; ++c) {
                    comps[c].id = s[6 + 3 * c];
                    comps[c].h = s[7 + 3 * c] >> 4;
                    comps[c].v = s[7 + 3 * c] & 15;
                    comps[c].tq = s[8 + 3 * c] & 3;
                    if (comps[c].h < 1 || comps[c].h > 4 || comps[c].v < 1 || comps[c].v > 4) {
                        err = "bad JPEG sampling factors";
                        return false;
                    }
                    hmax = std::max(hmax, comps[c].h);
                    vmax = std::max(vmax, comps[c].v);
                }
                const int mx = (W + 8 * hmax - 1) / (8 * hmax), my = (H + 8 * vmax - 1) / (8 * vmax);
                for (auto &c : comps) {
                    c.bw = mx * c.h;
                    c.bh = my * c.v;
                    c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
                }
                frame = true;
                break;
            }
            case 0xC2:
            case 0xC3:
            case 0xC5:
            case 0xC6:
            case 0xC7:
            case 0xC9:
            case 0xCA:
            case 0xCB:
            case 0xCD:
            case 0xCE:
            case 0xCF:
                err = "progressive, lossless or arithmetic-coded JPEG images are not decoded";
                return false;
            case 0xC4: {  // DHT
                size_t i = 0;
                while (i < sl) {
                    if (i + 17 > sl) {
                        err = "bad DHT";
                        return false;
                    }
                    const int tc = s[i] >> 4, th = s[i] & 3;
                    const uint8_t *counts = s + i + 1;
                    int total = 0;
                    for (int l = 0; l < 16; ++l) total += counts[l];
                    if (i + 17 + (size_t)total > sl || !(tc ? ac[th] : dc[th]).build(counts, s + i + 17, total)) {
                        err = "bad DHT";
                        return false;
                    }
                    i += 17 + (size_t)total;
                }
                break;
            }
            case 0xDD:  // DRI
                if (sl >= 2) restart = be16(s);
                break;
            case 0xDA: {  // SOS: one scan with every component (interleaved) or one component
                if (!frame || sl < 1) {
                    err = "scan before frame header";
                    return false;
                }
                const int ns = s[0];
                if (sl < 1 + 2 * (size_t)ns + 3 || ns < 1) {
                    err = "bad SOS";
                    return false;
                }
                std::vector<Comp *> sc;
                for (int k = 0; k < ns; ++k) {
                    Comp *c = nullptr;
                    for (auto &cc : comps)
                        if (cc.id == s[1 + 2 * k]) c = &cc;
                    if (!c) {
                        err = "scan names an unknown component";
                        return false;
                    }
                    c->td = s[2 + 2 * k] >> 4 & 3;
                    c->ta = s[2 + 2 * k] & 3;
                    c->pred = 0;
                    if (!dc[c->td].set || !ac[c->ta].set) {
                        err = "scan uses an undefined Huffman table";
                        return false;
                    }
                    sc.push_back(c);
                }
                Bits b{d, n, pos + len};
                float blk[64];
                int coef[64];
                auto block = [&](Comp &c, int bx, int by) -> bool {
                    memset(coef, 0, sizeof coef);
                    const int t = decode_sym(b, dc[c.td]);
                    if (t < 0 || t > 11) return false;
                    c.pred += extend(b.bits(t), t);
                    coef[0] = c.pred * q[c.tq][0];
                    for (int k = 1; k < 64;) {
                        const int rs = decode_sym(b, ac[c.ta]);
                        if (rs < 0) return false;
                        const int r = rs >> 4, sz = rs & 15;
                        if (sz == 0) {
                            if (r != 15) break;  // end of block
                            k += 16;
                            continue;
                        }
                        k += r;
                        if (k > 63) return false;
                        coef[kZigzag[k]] = extend(b.bits(sz), sz) * q[c.tq][k];
                        ++k;
                    }
                    for (int i = 0; i < 64; ++i) blk[i] = (float)coef[i];
                    idct8x8(blk, &c.plane[(size_t)by * 8 * c.bw * 8 + (size_t)bx * 8], c.bw * 8);
                    return true;
                };
                const bool inter = ns > 1;
                const int mx = (W + 8 * hmax - 1) / (8 * hmax), my = (H + 8 * vmax - 1) / (8 * vmax);
                // a single-component scan covers that component's own block grid
                const int cw = (W * sc[0]->h + hmax - 1) / hmax, ch = (H * sc[0]->v + vmax - 1) / vmax;
                const int ux = inter ? mx : (cw + 7) / 8, uy = inter ? my : (ch + 7) / 8;
                int count = 0;
                for (int y = 0; y < uy; ++y)
                    for (int x = 0; x < ux; ++x) {
                        if (restart && count == restart) {
                            b.restart();
                            for (Comp *c : sc) c->pred = 0;
                            count = 0;
                        }
                        ++count;
                        bool ok = true;
                        if (inter) {
                            for (Comp *c : sc)
                                for (int v = 0; v < c->v && ok; ++v)
                                    for (int h = 0; h < c->h && ok; ++h) ok = block(*c, x * c->h + h, y * c->v + v);
                        } else {
                            ok = block(*sc[0], x, y);
                        }
                        if (!ok) {
                            err = "corrupt JPEG image data";
                            return false;
                        }
                    }
                // continue after the entropy-coded data
                pos = b.pos;
                while (pos + 1 < n && !(d[pos] == 0xFF && d[pos + 1] != 0x00 && !(d[pos + 1] >= 0xD0 && d[pos + 1] <= 0xD7)))
                    ++pos;
                if (comps.size() == 1 || ns == (int)comps.size()) done = true;
                continue;
            }
            default:
                break;  // APPn, COM and others: skipped
        }
        pos += len;
    }
    if (!frame || comps.empty()) {
        err = "JPEG without image data";
        return false;
    }
    rgba.assign((size_t)W * H * 4, 255);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float s[3];
            for (size_t c = 0; c < comps.size(); ++c) {
                const Comp &cp = comps[c];
                const int sx = x * cp.h / hmax, sy = y * cp.v / vmax;  // chroma replication
                s[c] = cp.plane[(size_t)sy * cp.bw * 8 + sx];
            }
            uint8_t *o = &rgba[4 * ((size_t)y * W + x)];
            if (comps.size() == 1) {
                o[0] = o[1] = o[2] = (uint8_t)s[0];
            } else {
                const float Y = s[0], cb = s[1] - 128.0f, cr = s[2] - 128.0f;
                const float rgb[3] = {Y + 1.402f * cr, Y - 0.344136f * cb - 0.714136f * cr, Y + 1.772f * cb};
                for (int k = 0; k < 3; ++k) {
                    const float v = roundf(rgb[k]);
                    o[k] = (uint8_t)(v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v));
                }
            }
        }
    width = (uint32_t)W;
    height = (uint32_t)H;
    return true;
}

}  // namespace pg
