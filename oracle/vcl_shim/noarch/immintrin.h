// immintrin.h stand-in - TEST INFRASTRUCTURE: see xmmintrin.h beside it.
#pragma once
#include "xmmintrin.h"
