// Minimal stand-in for the parts of the GLM vector library that the vendored
// lightpmm headers use (glm is not installed in this image).  Test
// infrastructure only: it lets oracle/lightpmm_harness.cpp compile the
// reference's own lightpmm code where it lies; nothing in the product links it.
#pragma once
#include <cmath>
#include <cstddef>

namespace glm {

struct vec3 {
    float x, y, z;
    vec3() : x(0.f), y(0.f), z(0.f) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float &operator[](std::size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float &operator[](std::size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3 operator+(const vec3 &o) const { return {x + o.x, y + o.y, z + o.z}; }
    vec3 operator-(const vec3 &o) const { return {x - o.x, y - o.y, z - o.z}; }
    vec3 operator*(const vec3 &o) const { return {x * o.x, y * o.y, z * o.z}; }
    vec3 operator*(float s) const { return {x * s, y * s, z * s}; }
    vec3 operator/(float s) const { return {x / s, y / s, z / s}; }
    vec3 operator-() const { return {-x, -y, -z}; }
    vec3 &operator+=(const vec3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3 &operator-=(const vec3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3 &operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3 &operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
    bool operator==(const vec3 &o) const { return x == o.x && y == o.y && z == o.z; }
    // GLM's member length() is the number of components, not the Euclidean
    // norm (glm::length is); code that calls it gets 3, as with the real library
    static constexpr int length() { return 3; }
};
inline vec3 operator*(float s, const vec3 &v) { return v * s; }

inline float dot(const vec3 &a, const vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3 &a, const vec3 &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3 &v) { return v * (1.0f / length(v)); }

}  // namespace glm
