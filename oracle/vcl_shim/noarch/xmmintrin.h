// xmmintrin.h / immintrin.h stand-in - TEST INFRASTRUCTURE, for hosts without
// x86 SSE (the Arm host).  The reference's lightpmm headers include these and
// define one helper over SSE types (my_fastpow2 in pmm-vcl.h, not called by the
// fit); this gives those types and operations lane loops so the headers build.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

struct __m128 {
    float f[4];
};
struct __m128i {
    int32_t i[4];
};
#define _MM_FROUND_TO_ZERO 3
// denormal modes: the SSE control-register switches have no counterpart here;
// the modes stay as the host's floating-point environment sets them
#define _MM_FLUSH_ZERO_ON 0x8000
#define _MM_FLUSH_ZERO_OFF 0x0000
#define _MM_DENORMALS_ZERO_ON 0x0040
#define _MM_DENORMALS_ZERO_OFF 0x0000
#define _MM_SET_FLUSH_ZERO_MODE(mode) ((void)(mode))
#define _MM_SET_DENORMALS_ZERO_MODE(mode) ((void)(mode))

static inline __m128 _mm_set1_ps(float a) { return __m128{{a, a, a, a}}; }
#define PG_SSE_BIN(name, expr)                                   \
    static inline __m128 name(__m128 a, __m128 b) {              \
        __m128 r;                                                \
        for (int k = 0; k < 4; ++k) r.f[k] = (expr);             \
        return r;                                                \
    }
PG_SSE_BIN(_mm_add_ps, a.f[k] + b.f[k])
PG_SSE_BIN(_mm_sub_ps, a.f[k] - b.f[k])
PG_SSE_BIN(_mm_mul_ps, a.f[k] * b.f[k])
PG_SSE_BIN(_mm_div_ps, a.f[k] / b.f[k])
PG_SSE_BIN(_mm_max_ps, a.f[k] > b.f[k] ? a.f[k] : b.f[k])
#undef PG_SSE_BIN
static inline __m128 _mm_round_ps(__m128 a, int) {
    __m128 r;
    for (int k = 0; k < 4; ++k) r.f[k] = std::trunc(a.f[k]);
    return r;
}
static inline __m128i _mm_cvtps_epi32(__m128 a) {
    __m128i r;
    for (int k = 0; k < 4; ++k) r.i[k] = (int32_t)std::nearbyint(a.f[k]);
    return r;
}
static inline __m128 _mm_castsi128_ps(__m128i a) {
    __m128 r;
    std::memcpy(r.f, a.i, sizeof r.f);
    return r;
}
