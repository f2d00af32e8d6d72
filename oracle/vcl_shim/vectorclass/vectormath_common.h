// vectormath_common.h - TEST INFRASTRUCTURE.  Natural logarithm of the
// portable vectorclass stand-in (vectorclass.h): per lane, x = m 2^e with m in
// [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) with s = (m - 1) / (m + 1), the
// odd series of atanh to s^9 (|s| <= 0.172, truncation below 3e-9 relative),
// log x = e ln 2 + log m; negative and NaN inputs give NaN, 0 gives -inf,
// +inf gives +inf, subnormals are scaled first.  Branch-free in the common
// path so the lane loop vectorises.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

namespace vcl {

inline float log_lane(float x) {
    if (!(x > 0.0f) || std::isinf(x)) {
        if (x == 0.0f) return -std::numeric_limits<float>::infinity();
        if (std::isinf(x) && x > 0.0f) return x;
        return std::numeric_limits<float>::quiet_NaN();
    }
    int e = 0;
    if (x < 1.17549435e-38f) {  // subnormal: scale by 2^23
        x *= 8388608.0f;
        e = -23;
    }
    uint32_t u;
    std::memcpy(&u, &x, sizeof u);
    e += (int)((u >> 23) & 0xffu) - 127;
    u = (u & 0x007fffffu) | 0x3f800000u;
    float m;
    std::memcpy(&m, &u, sizeof m);
    if (m > 1.41421356f) {
        m *= 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f), s2 = s * s;
    const float series = s2 * (1.0f / 3.0f + s2 * (1.0f / 5.0f + s2 * (1.0f / 7.0f + s2 * (1.0f / 9.0f))));
    const float lm = 2.0f * s + 2.0f * s * series;
    return (float)e * 0.693147182f + lm;
}

template <int N>
inline VecFloat<N> log(const VecFloat<N> &a) {
    VecFloat<N> r;
    for (int i = 0; i < N; ++i) r.v[i] = log_lane(a.v[i]);
    return r;
}

}  // namespace vcl
