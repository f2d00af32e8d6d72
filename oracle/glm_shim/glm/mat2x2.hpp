// Minimal GLM stand-in (column-major 2x2 matrix) for compiling the vendored
// lightpmm headers in the oracle harness.  Test infrastructure only.
#pragma once
#include "vec2.hpp"

namespace glm {

struct mat2x2 {
    vec2 c[2];
    mat2x2() : c{vec2(1.f, 0.f), vec2(0.f, 1.f)} {}
    explicit mat2x2(float s) : c{vec2(s, 0.f), vec2(0.f, s)} {}
    mat2x2(const vec2 &a, const vec2 &b) : c{a, b} {}
    mat2x2(float x0, float y0, float x1, float y1) : c{vec2(x0, y0), vec2(x1, y1)} {}
    vec2 &operator[](std::size_t i) { return c[i]; }
    const vec2 &operator[](std::size_t i) const { return c[i]; }
};

}  // namespace glm
