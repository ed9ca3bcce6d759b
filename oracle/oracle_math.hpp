// oracle_math.hpp — scalar layer of the MM3E CPU-path oracle.
//
// TEST INFRASTRUCTURE ONLY. The oracle is the parity checker for the CUDA render path and the
// timed CPU baseline; nothing in the shipped library links or calls it.
//
// The reference is Rust `f32` code. This header reproduces the Rust scalar semantics the render
// path relies on, for any scalar type T (float = the oracle proper, double = the FP64
// re-march, CountF = the operation counter):
//   * `f32::max`/`f32::min` ignore a NaN operand (LLVM maxnum/minnum) -> fmax/fmin;
//   * `f32::clamp` is `if x < lo {lo}; if x > hi {hi}` (NaN passes through);
//   * `f32::signum` returns +-1 for +-0 and NaN for NaN;
//   * `f32::fract` is `x - trunc(x)`; `f32::round` is half away from zero (roundf);
//   * `powi(n)` with a constant n is expanded by LLVM into square-and-multiply;
//   * `f32 as i32` saturates and maps NaN to 0.
// Transcendentals (sin, cos, tan, exp, powf, acos) call the platform libm, which is what Rust's
// `f32` methods lower to on Linux.
#pragma once
#include <cmath>
#include <cstdint>
#include <limits>

namespace oracle {

// ---- literals: parse decimal constants straight to the scalar type (no double rounding) ----
template <class T> struct Lit;
template <> struct Lit<float> { static float get(float f, double) { return f; } };
template <> struct Lit<double> { static double get(float, double d) { return d; } };
#define OL(x) (::oracle::Lit<T>::get(x##f, x))

// ---- float / double overloads ----
inline float o_sqrt(float x) { return std::sqrt(x); }
inline double o_sqrt(double x) { return std::sqrt(x); }
inline float o_sin(float x) { return ::sinf(x); }
inline double o_sin(double x) { return std::sin(x); }
inline float o_cos(float x) { return ::cosf(x); }
inline double o_cos(double x) { return std::cos(x); }
inline float o_tan(float x) { return ::tanf(x); }
inline double o_tan(double x) { return std::tan(x); }
inline float o_exp(float x) { return ::expf(x); }
inline double o_exp(double x) { return std::exp(x); }
inline float o_pow(float x, float y) { return ::powf(x, y); }
inline double o_pow(double x, double y) { return std::pow(x, y); }
inline float o_acos(float x) { return ::acosf(x); }
inline double o_acos(double x) { return std::acos(x); }
inline float o_floor(float x) { return ::floorf(x); }
inline double o_floor(double x) { return std::floor(x); }
inline float o_round(float x) { return ::roundf(x); }
inline double o_round(double x) { return std::round(x); }
inline float o_trunc(float x) { return ::truncf(x); }
inline double o_trunc(double x) { return std::trunc(x); }
inline float o_abs(float x) { return std::fabs(x); }
inline double o_abs(double x) { return std::fabs(x); }
inline float o_max(float a, float b) { return std::fmax(a, b); }
inline double o_max(double a, double b) { return std::fmax(a, b); }
inline float o_min(float a, float b) { return std::fmin(a, b); }
inline double o_min(double a, double b) { return std::fmin(a, b); }
inline bool o_isfinite(float x) { return std::isfinite(x); }
inline bool o_isfinite(double x) { return std::isfinite(x); }
inline bool o_isnan(float x) { return std::isnan(x); }
inline bool o_isnan(double x) { return std::isnan(x); }
inline double o_value(float x) { return x; }
inline double o_value(double x) { return x; }

// Rust `f32::clamp` (core::f32::clamp): sequential compares, NaN passes through.
template <class T> inline T o_clamp(T x, T lo, T hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
// Rust `f32::signum`.
template <class T> inline T o_signum(T x) {
    if (o_isnan(x)) return x;
    return std::signbit(o_value(x)) ? T(-1) : T(1);
}
// Rust `f32::fract`.
template <class T> inline T o_fract(T x) { return x - o_trunc(x); }
// Rust `x.powi(5)`: LLVM square-and-multiply, x * ((x*x)*(x*x)).
template <class T> inline T o_powi5(T x) {
    T x2 = x * x;
    T x4 = x2 * x2;
    return x * x4;
}
// Rust `f32 as i32` (saturating, NaN -> 0).
template <class T> inline int32_t o_to_i32(T x) {
    double v = o_value(x);
    if (std::isnan(v)) return 0;
    if (v >= 2147483647.0) return INT32_MAX;
    if (v <= -2147483648.0) return INT32_MIN;
    return (int32_t)v;
}
// Rust `f32 as usize` (saturating, NaN -> 0, negatives -> 0).
template <class T> inline uint64_t o_to_usize(T x) {
    double v = o_value(x);
    if (std::isnan(v) || v <= 0.0) return 0;
    if (v >= 18446744073709551615.0) return UINT64_MAX;
    return (uint64_t)v;
}

template <class T> inline T o_inf() { return T(std::numeric_limits<float>::infinity()); }

// Render phases the counting instantiation attributes work to.
// The first four are the primary level's; the *_REFL phases are the reflection levels' passes.
enum : int {
    PH_MARCH = 0, PH_AO = 1, PH_SHADOW = 2, PH_SHADE = 3,
    PH_MARCH_REFL = 4, PH_AO_REFL = 5, PH_SHADOW_REFL = 6, PH_COUNT = 7
};

// Event hooks for the counting instantiation (no-ops for float / double).
template <class T> struct Hooks {
    static int phase(int) { return PH_SHADE; }
    static void field_eval() {}
    static void dual_eval() {}
    static void primary_ray() {}
    static void reflection_ray() {}
    static void shadow_ray() {}
    static void gi_ray() {}
};

// Attributes the work of a scope to a render phase (counting instantiation only).
template <class T> struct PhaseScope {
    int prev;
    explicit PhaseScope(int ph) : prev(Hooks<T>::phase(ph)) {}
    ~PhaseScope() { Hooks<T>::phase(prev); }
};

}  // namespace oracle
