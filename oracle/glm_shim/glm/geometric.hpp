// Minimal GLM stand-in: geometric functions live in vec3.hpp.  Test infrastructure only.
#pragma once
#include "vec2.hpp"
#include "vec3.hpp"
