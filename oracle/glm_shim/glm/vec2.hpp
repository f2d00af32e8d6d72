// Minimal GLM stand-in (2-vector) for compiling the vendored lightpmm headers
// in the oracle harness.  Test infrastructure only.
#pragma once
#include <cmath>
#include <cstddef>

namespace glm {

struct vec2 {
    float x, y;
    vec2() : x(0.f), y(0.f) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    float &operator[](std::size_t i) { return i == 0 ? x : y; }
    const float &operator[](std::size_t i) const { return i == 0 ? x : y; }
    vec2 operator+(const vec2 &o) const { return {x + o.x, y + o.y}; }
    vec2 operator-(const vec2 &o) const { return {x - o.x, y - o.y}; }
    vec2 operator*(float s) const { return {x * s, y * s}; }
    vec2 &operator*=(float s) { x *= s; y *= s; return *this; }
    bool operator==(const vec2 &o) const { return x == o.x && y == o.y; }
};
inline vec2 operator*(float s, const vec2 &v) { return v * s; }
inline float dot(const vec2 &a, const vec2 &b) { return a.x * b.x + a.y * b.y; }

}  // namespace glm
