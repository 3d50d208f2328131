// C99 cabs() for the reference's ptychography driver (util/ptycho.cpp uses it
// on a complexFormat), which a C++ translation unit does not declare.
#pragma once
#include <cmath>
inline double cabs(complexFormat z) { return std::hypot((double)crealf(z), (double)cimagf(z)); }
