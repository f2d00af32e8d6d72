// vectormath_exp.h - TEST INFRASTRUCTURE: the portable vectorclass stand-in's
// logarithm (vectormath_common.h); lightpmm takes exp from its own fastexp.
#pragma once
#include "vectorclass.h"
