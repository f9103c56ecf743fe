// Force-included before the reference's headers for the ref_driver_fabs
// build: brings the floating-point overloads of abs into the global
// namespace, so the reference's unqualified abs(double) calls
// (interpolation.h:199-200) compare real distances instead of truncated ints.
#pragma once
#include <cmath>
#include <cstdlib>
using std::abs;
