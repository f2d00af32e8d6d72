// vectormath_hyp.h - TEST INFRASTRUCTURE: the portable vectorclass stand-in;
// lightpmm takes tanh from its own fasttanh.
#pragma once
#include "vectorclass.h"
