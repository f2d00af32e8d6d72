// vectorclass.h - TEST INFRASTRUCTURE.  A portable stand-in for the subset of
// Agner Fog's vectorclass library that the reference's vendored lightpmm uses
// (external/lightpmm/include/pmm/pmm-vcl.h and the lightpmm headers): float
// vectors of 4 and 8 lanes, their boolean masks and integer vectors, the
// element-wise operators, selection, horizontal reductions and the few math
// functions.  Each operation is a plain loop over the lanes in IEEE single
// precision, so it builds on any host (the reference's SIMD back ends are x86
// only) and the compiler may vectorise it.  Written for this project from the
// library's documented interface; oracle/build_oracle.py puts this directory
// ahead of the vendored library only where that library cannot build.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace vcl {

template <int N>
struct VecMask {
    bool m[N];
    VecMask() {
        for (int i = 0; i < N; ++i) m[i] = false;
    }
    VecMask(bool b) {
        for (int i = 0; i < N; ++i) m[i] = b;
    }
    bool operator[](int i) const { return m[i]; }
    bool extract(int i) const { return m[i]; }
    VecMask &insert(int i, bool b) {
        m[i] = b;
        return *this;
    }
};

template <int N>
struct VecInt {
    int32_t v[N];
    int32_t operator[](int i) const { return v[i]; }
};

template <int N>
struct VecFloat {
    float v[N];
    VecFloat() {
        for (int i = 0; i < N; ++i) v[i] = 0.0f;
    }
    VecFloat(float s) {
        for (int i = 0; i < N; ++i) v[i] = s;
    }
    VecFloat(float a, float b, float c, float d) {
        static_assert(N == 4, "four values for a four-lane vector");
        v[0] = a;
        v[1] = b;
        v[2] = c;
        v[3] = d;
    }
    VecFloat(float a, float b, float c, float d, float e, float f, float g, float h) {
        static_assert(N == 8, "eight values for an eight-lane vector");
        v[0] = a;
        v[1] = b;
        v[2] = c;
        v[3] = d;
        v[4] = e;
        v[5] = f;
        v[6] = g;
        v[7] = h;
    }
    float operator[](int i) const { return v[i]; }
    float extract(int i) const { return v[i]; }
    VecFloat &insert(int i, float x) {
        v[i] = x;
        return *this;
    }
    VecFloat &load(const float *p) {
        for (int i = 0; i < N; ++i) v[i] = p[i];
        return *this;
    }
    void store(float *p) const {
        for (int i = 0; i < N; ++i) p[i] = v[i];
    }
    static constexpr int size() { return N; }
    // lanes from n on set to zero
    VecFloat &cutoff(int n) {
        for (int i = n < 0 ? 0 : n; i < N; ++i) v[i] = 0.0f;
        return *this;
    }
    VecFloat &operator+=(const VecFloat &o) {
        for (int i = 0; i < N; ++i) v[i] += o.v[i];
        return *this;
    }
    VecFloat &operator-=(const VecFloat &o) {
        for (int i = 0; i < N; ++i) v[i] -= o.v[i];
        return *this;
    }
    VecFloat &operator*=(const VecFloat &o) {
        for (int i = 0; i < N; ++i) v[i] *= o.v[i];
        return *this;
    }
    VecFloat &operator/=(const VecFloat &o) {
        for (int i = 0; i < N; ++i) v[i] /= o.v[i];
        return *this;
    }
};

typedef VecFloat<4> Vec4f;
typedef VecFloat<8> Vec8f;
typedef VecMask<4> Vec4fb;
typedef VecMask<8> Vec8fb;
typedef VecInt<4> Vec4i;
typedef VecInt<8> Vec8i;

#define PG_VCL_BINARY(op)                                                                 \
    template <int N>                                                                      \
    inline VecFloat<N> operator op(const VecFloat<N> &a, const VecFloat<N> &b) {          \
        VecFloat<N> r;                                                                    \
        for (int i = 0; i < N; ++i) r.v[i] = a.v[i] op b.v[i];                             \
        return r;                                                                         \
    }                                                                                     \
    template <int N>                                                                      \
    inline VecFloat<N> operator op(const VecFloat<N> &a, float b) {                       \
        return a op VecFloat<N>(b);                                                       \
    }                                                                                     \
    template <int N>                                                                      \
    inline VecFloat<N> operator op(float a, const VecFloat<N> &b) {                       \
        return VecFloat<N>(a) op b;                                                       \
    }
PG_VCL_BINARY(+)
PG_VCL_BINARY(-)
PG_VCL_BINARY(*)
PG_VCL_BINARY(/)
#undef PG_VCL_BINARY

template <int N>
inline VecFloat<N> operator-(const VecFloat<N> &a) {
    VecFloat<N> r;
    for (int i = 0; i < N; ++i) r.v[i] = -a.v[i];
    return r;
}

#define PG_VCL_COMPARE(op)                                                                \
    template <int N>                                                                      \
    inline VecMask<N> operator op(const VecFloat<N> &a, const VecFloat<N> &b) {           \
        VecMask<N> r;                                                                     \
        for (int i = 0; i < N; ++i) r.m[i] = a.v[i] op b.v[i];                             \
        return r;                                                                         \
    }                                                                                     \
    template <int N>                                                                      \
    inline VecMask<N> operator op(const VecFloat<N> &a, float b) {                        \
        return a op VecFloat<N>(b);                                                       \
    }                                                                                     \
    template <int N>                                                                      \
    inline VecMask<N> operator op(float a, const VecFloat<N> &b) {                        \
        return VecFloat<N>(a) op b;                                                       \
    }
PG_VCL_COMPARE(<)
PG_VCL_COMPARE(<=)
PG_VCL_COMPARE(>)
PG_VCL_COMPARE(>=)
PG_VCL_COMPARE(==)
PG_VCL_COMPARE(!=)
#undef PG_VCL_COMPARE

#define PG_VCL_LOGIC(op)                                                                  \
    template <int N>                                                                      \
    inline VecMask<N> operator op(const VecMask<N> &a, const VecMask<N> &b) {             \
        VecMask<N> r;                                                                     \
        for (int i = 0; i < N; ++i) r.m[i] = a.m[i] op b.m[i];                             \
        return r;                                                                         \
    }
#define PG_VCL_LOGIC_SCALAR(op)                                                           \
    template <int N>                                                                      \
    inline VecMask<N> operator op(bool a, const VecMask<N> &b) {                          \
        return VecMask<N>(a) op b;                                                        \
    }                                                                                     \
    template <int N>                                                                      \
    inline VecMask<N> operator op(const VecMask<N> &a, bool b) {                          \
        return a op VecMask<N>(b);                                                        \
    }
PG_VCL_LOGIC(&)
PG_VCL_LOGIC(|)
PG_VCL_LOGIC(^)
PG_VCL_LOGIC(&&)
PG_VCL_LOGIC(||)
PG_VCL_LOGIC(==)
PG_VCL_LOGIC(!=)
#undef PG_VCL_LOGIC
PG_VCL_LOGIC_SCALAR(&)
PG_VCL_LOGIC_SCALAR(|)
PG_VCL_LOGIC_SCALAR(&&)
PG_VCL_LOGIC_SCALAR(||)
#undef PG_VCL_LOGIC_SCALAR

// a float vector used as a condition: lanes equal to zero
template <int N>
inline VecMask<N> operator!(const VecFloat<N> &a) {
    VecMask<N> r;
    for (int i = 0; i < N; ++i) r.m[i] = a.v[i] == 0.0f;
    return r;
}

template <int N>
inline VecMask<N> operator!(const VecMask<N> &a) {
    VecMask<N> r;
    for (int i = 0; i < N; ++i) r.m[i] = !a.m[i];
    return r;
}
template <int N>
inline VecMask<N> operator~(const VecMask<N> &a) {
    return !a;
}
template <int N>
inline VecMask<N> &operator&=(VecMask<N> &a, const VecMask<N> &b) {
    a = a & b;
    return a;
}
template <int N>
inline VecMask<N> &operator|=(VecMask<N> &a, const VecMask<N> &b) {
    a = a | b;
    return a;
}

template <int N>
inline bool horizontal_and(const VecMask<N> &a) {
    for (int i = 0; i < N; ++i)
        if (!a.m[i]) return false;
    return true;
}
template <int N>
inline bool horizontal_or(const VecMask<N> &a) {
    for (int i = 0; i < N; ++i)
        if (a.m[i]) return true;
    return false;
}
// lanes summed pairwise, as a two-level shuffle-and-add reduction does
template <int N>
inline float horizontal_add(const VecFloat<N> &a) {
    float t[N];
    for (int i = 0; i < N; ++i) t[i] = a.v[i];
    for (int w = N / 2; w >= 1; w /= 2)
        for (int i = 0; i < w; ++i) t[i] = t[i] + t[i + w];
    return t[0];
}

template <int N>
inline VecFloat<N> select(const VecMask<N> &s, const VecFloat<N> &a, const VecFloat<N> &b) {
    VecFloat<N> r;
    for (int i = 0; i < N; ++i) r.v[i] = s.m[i] ? a.v[i] : b.v[i];
    return r;
}
template <int N>
inline VecFloat<N> select(const VecMask<N> &s, float a, const VecFloat<N> &b) {
    return select(s, VecFloat<N>(a), b);
}
template <int N>
inline VecFloat<N> select(const VecMask<N> &s, const VecFloat<N> &a, float b) {
    return select(s, a, VecFloat<N>(b));
}

#define PG_VCL_MAP(name, expr)                                                            \
    template <int N>                                                                      \
    inline VecFloat<N> name(const VecFloat<N> &a) {                                       \
        VecFloat<N> r;                                                                    \
        for (int i = 0; i < N; ++i) {                                                     \
            const float x = a.v[i];                                                       \
            r.v[i] = (expr);                                                              \
        }                                                                                 \
        return r;                                                                         \
    }
PG_VCL_MAP(sqrt, std::sqrt(x))
PG_VCL_MAP(abs, std::fabs(x))
PG_VCL_MAP(truncate, std::trunc(x))
#undef PG_VCL_MAP

template <int N>
inline VecFloat<N> min(const VecFloat<N> &a, const VecFloat<N> &b) {
    VecFloat<N> r;
    for (int i = 0; i < N; ++i) r.v[i] = a.v[i] < b.v[i] ? a.v[i] : b.v[i];
    return r;
}
template <int N>
inline VecFloat<N> max(const VecFloat<N> &a, const VecFloat<N> &b) {
    VecFloat<N> r;
    for (int i = 0; i < N; ++i) r.v[i] = a.v[i] > b.v[i] ? a.v[i] : b.v[i];
    return r;
}

#define PG_VCL_CLASS(name, expr)                                                          \
    template <int N>                                                                      \
    inline VecMask<N> name(const VecFloat<N> &a) {                                        \
        VecMask<N> r;                                                                     \
        for (int i = 0; i < N; ++i) r.m[i] = (expr)(a.v[i]);                               \
        return r;                                                                         \
    }
PG_VCL_CLASS(is_finite, std::isfinite)
PG_VCL_CLASS(is_inf, std::isinf)
PG_VCL_CLASS(is_nan, std::isnan)
#undef PG_VCL_CLASS

// nearest integer, ties to even (the default rounding mode)
template <int N>
inline VecInt<N> roundi(const VecFloat<N> &a) {
    VecInt<N> r;
    for (int i = 0; i < N; ++i) r.v[i] = (int32_t)std::nearbyint(a.v[i]);
    return r;
}
template <int N>
inline VecFloat<N> reinterpret_f(const VecInt<N> &a) {
    VecFloat<N> r;
    std::memcpy(r.v, a.v, sizeof(r.v));
    return r;
}
// a * b + c with two roundings (the reference builds without FMA instructions)
template <int N>
inline VecFloat<N> mul_add(const VecFloat<N> &a, const VecFloat<N> &b, const VecFloat<N> &c) {
    return a * b + c;
}
// c0 + c1 x + c2 x^2 + c3 x^3 + c4 x^4
template <int N>
inline VecFloat<N> polynomial_4(const VecFloat<N> &x, float c0, float c1, float c2, float c3, float c4) {
    return mul_add(mul_add(mul_add(mul_add(VecFloat<N>(c4), x, VecFloat<N>(c3)), x, VecFloat<N>(c2)), x,
                           VecFloat<N>(c1)),
                   x, VecFloat<N>(c0));
}
// the magnitude of a with the sign of b
template <int N>
inline VecFloat<N> sign_combine(const VecFloat<N> &a, const VecFloat<N> &b) {
    VecFloat<N> r;
    for (int i = 0; i < N; ++i) r.v[i] = std::signbit(b.v[i]) ? -a.v[i] : a.v[i];
    return r;
}

}  // namespace vcl

#include "vectormath_common.h"
