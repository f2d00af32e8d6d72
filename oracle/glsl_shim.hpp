// glsl_shim.hpp - TEST INFRASTRUCTURE.  The subset of GLSL 4.60 that the
// reference's shader functions use, as C++ in FP32, so that their bodies
// compile as host code: vec2/vec3/vec4 with GLSL's component-wise operators
// and constructors, the built-in functions (dot, cross, normalize, length,
// reflect, refract, mix, clamp, the float math functions with GLSL's
// argument conventions: atan(y, x), pow/exp/log/sqrt in single precision),
// `uint`, and a helper for the scalar swizzle `.xxx`.
//
// Everything lives in namespace glsl so that the unqualified calls in the
// shader text resolve to these single-precision overloads and never to the
// C library's double functions.  Used only by oracle/build_glsl_ref.py,
// which includes the shader text after this header.
#pragma once

#include <cmath>
#include <cstdint>

#undef M_PI
#undef M_2PI
#undef E

namespace glsl {

typedef uint32_t uint;

struct vec2 {
    float x, y;
    vec2() : x(0.0f), y(0.0f) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
    float x, y, z;
    vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3 &operator+=(const vec3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3 &operator-=(const vec3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3 &operator*=(const vec3 &o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    vec3 &operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3 &operator/=(const vec3 &o) { x /= o.x; y /= o.y; z /= o.z; return *this; }
    vec3 &operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

struct vec4 {
    float x, y, z, w;
    vec3 xyz;  // kept equal to (x, y, z): vec4 values are only built and read here
    vec4() : x(0), y(0), z(0), w(0), xyz() {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s), xyz(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d), xyz(a, b, c) {}
    vec4(const vec3 &v, float d) : x(v.x), y(v.y), z(v.z), w(d), xyz(v) {}
};

struct ivec3 {
    int x, y, z;
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
};

struct mat4 {
    float m[16];  // column-major, as GLSL: m[4 * column + row]
};
inline vec4 operator*(const mat4 &a, const vec4 &v) {
    float r[4];
    for (int i = 0; i < 4; ++i) r[i] = a.m[i] * v.x + a.m[4 + i] * v.y + a.m[8 + i] * v.z + a.m[12 + i] * v.w;
    return vec4(r[0], r[1], r[2], r[3]);
}

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator+(vec3 a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }

// scalar functions, single precision as in GLSL
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float sqrt(float x) { return std::sqrt(x); }
inline float exp(float x) { return std::exp(x); }
inline float log(float x) { return std::log(x); }
inline float pow(float a, float b) { return std::pow(a, b); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float tan(float x) { return std::tan(x); }
inline float acos(float x) { return std::acos(x); }
inline float atan(float x) { return std::atan(x); }
inline float atan(float y, float x) { return std::atan2(y, x); }
inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }

// geometric functions
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(vec3 a) { return sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }
inline vec3 reflect(vec3 i, vec3 n) { return i - 2.0f * dot(n, i) * n; }
inline vec3 refract(vec3 i, vec3 n, float eta) {
    const float k = 1.0f - eta * eta * (1.0f - dot(n, i) * dot(n, i));
    if (k < 0.0f) return vec3(0.0f);
    return eta * i - (eta * dot(n, i) + sqrt(k)) * n;
}
inline vec3 abs(vec3 a) { return vec3(abs(a.x), abs(a.y), abs(a.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 mix(vec3 a, vec3 b, float t) { return a * (1.0f - t) + b * t; }

// atomicAdd on a buffer member: the old value (the tests run the cache's
// create / update functions on one thread)
inline uint atomicAdd(uint &x, uint v) {
    const uint old = x;
    x += v;
    return old;
}

// `expr.xxx` of a scalar expression
inline vec3 xxx(float s) { return vec3(s); }

// Texture lookups: sampler 0 is the environment map (raytrace.rmiss,
// raytrace.rgen:406-421), answered by the estimator harness; the tests use
// untextured materials, so no other sampler is read.
extern int textureSamplers[64];
vec4 texture(int sampler, vec2 uv);

}  // namespace glsl
