// Host definitions of the CUDA device intrinsics that device_math.cuh uses, so that the world
// field (the tape interpreter and a scene-specialised program) compiles as plain C++ for a host
// comparison (tests/host_checks.py). Every definition is exact: bit reinterpretations,
// a correctly rounded fused multiply-add, an upward-rounded binary32 sum, a saturating
// truncation. Test infrastructure only.
#pragma once
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <math.h>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include <cuda_runtime.h>
// (Standard headers come before the __noinline__ stand-in below, which their attributes spell.)

inline float __int_as_float(int x) { float f; std::memcpy(&f, &x, 4); return f; }
inline float __uint_as_float(unsigned x) { float f; std::memcpy(&f, &x, 4); return f; }
inline int __float_as_int(float f) { int x; std::memcpy(&x, &f, 4); return x; }
inline unsigned __float_as_uint(float f) { unsigned x; std::memcpy(&x, &f, 4); return x; }
inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
// Rust `as i32`: truncation toward zero, saturating, NaN -> 0.
inline int __float2int_rz(float x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}
// Truncation toward zero to an unsigned integer, saturating, NaN -> 0.
inline unsigned __float2uint_rz(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 4294967295u;
    return (unsigned)x;
}
// fl_up(a + b): the binary64 sum and its exact error (Knuth's two-sum) pick the smallest binary32
// value at or above the exact sum.
inline float __fadd_ru(float a, float b) {
    const double s = (double)a + (double)b;
    const double bb = s - (double)a;
    const double err = ((double)a - (s - bb)) + ((double)b - bb);
    float f = (float)s;
    if (std::isfinite(s) && ((double)f < s || ((double)f == s && err > 0.0)))
        f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}
template <class T> inline T __ldg(const T* p) { return *p; }
using std::isfinite;
using std::isnan;
using std::signbit;
#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif
#ifndef __grid_constant__
#define __grid_constant__
#endif
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif
inline uint32_t min(uint32_t a, uint32_t b) { return a < b ? a : b; }
inline uint32_t max(uint32_t a, uint32_t b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
