// oracle_count.hpp — an operation-counting f32 scalar for the oracle.
//
// TEST / MEASUREMENT INFRASTRUCTURE ONLY. Instantiating the oracle with CountF renders exactly
// what the float oracle renders (every operation is evaluated in f32) while counting the
// algorithmic work. The counts are the roofline numerator of the CUDA path:
//   fp32  = add + sub + mul + min/max + compare-select   (an FMA on the GPU retires two of these)
//   div, sqrt and transcendentals (sin/cos/tan/exp/pow/acos) are counted separately and are not
//   part of the FP32-pipe numerator.
// Counters are thread-local; the render driver sums them over worker threads. They are kept per
// render phase (PH_MARCH: march + hit normal, PH_AO, PH_SHADOW, each for the primary level and
// for the reflection levels, PH_SHADE: everything else), matching the kernels the CUDA path
// splits a frame into.
#pragma once
#include <cstdint>

#include "oracle_math.hpp"

namespace oracle {

struct OpCounts {
    uint64_t add = 0, mul = 0, cmp = 0, minmax = 0, div = 0, sqrt = 0, trans = 0;
    uint64_t field_evals = 0, dual_evals = 0;
    uint64_t primary_rays = 0, reflection_rays = 0, shadow_rays = 0, gi_rays = 0;
    void merge(const OpCounts& o) {
        add += o.add; mul += o.mul; cmp += o.cmp; minmax += o.minmax; div += o.div; sqrt += o.sqrt;
        trans += o.trans; field_evals += o.field_evals; dual_evals += o.dual_evals;
        primary_rays += o.primary_rays; reflection_rays += o.reflection_rays;
        shadow_rays += o.shadow_rays; gi_rays += o.gi_rays;
    }
    uint64_t fp32() const { return add + mul + cmp + minmax; }
};

inline OpCounts* phase_counts() {
    static thread_local OpCounts c[PH_COUNT];
    return c;
}
inline int& current_phase() {
    static thread_local int ph = PH_SHADE;
    return ph;
}
inline OpCounts& op_counts() { return phase_counts()[current_phase()]; }
inline void reset_counts() {
    for (int i = 0; i < PH_COUNT; ++i) phase_counts()[i] = OpCounts();
    current_phase() = PH_SHADE;
}

struct CountF {
    float v;
    CountF() : v(0.0f) {}
    CountF(float x) : v(x) {}
    CountF(double x) : v((float)x) {}
    CountF(int x) : v((float)x) {}
    CountF(unsigned x) : v((float)x) {}
    CountF(long x) : v((float)x) {}
    CountF(unsigned long x) : v((float)x) {}
};

inline CountF operator+(CountF a, CountF b) { op_counts().add++; return CountF(a.v + b.v); }
inline CountF operator-(CountF a, CountF b) { op_counts().add++; return CountF(a.v - b.v); }
inline CountF operator*(CountF a, CountF b) { op_counts().mul++; return CountF(a.v * b.v); }
inline CountF operator/(CountF a, CountF b) { op_counts().div++; return CountF(a.v / b.v); }
inline CountF operator-(CountF a) { return CountF(-a.v); }
inline CountF& operator+=(CountF& a, CountF b) { a = a + b; return a; }
inline CountF& operator-=(CountF& a, CountF b) { a = a - b; return a; }
inline CountF& operator*=(CountF& a, CountF b) { a = a * b; return a; }
inline CountF& operator/=(CountF& a, CountF b) { a = a / b; return a; }
inline bool operator<(CountF a, CountF b) { op_counts().cmp++; return a.v < b.v; }
inline bool operator>(CountF a, CountF b) { op_counts().cmp++; return a.v > b.v; }
inline bool operator<=(CountF a, CountF b) { op_counts().cmp++; return a.v <= b.v; }
inline bool operator>=(CountF a, CountF b) { op_counts().cmp++; return a.v >= b.v; }
inline bool operator==(CountF a, CountF b) { op_counts().cmp++; return a.v == b.v; }
inline bool operator!=(CountF a, CountF b) { op_counts().cmp++; return a.v != b.v; }

template <> struct Hooks<CountF> {
    static void field_eval() { op_counts().field_evals++; }
    static void dual_eval() { op_counts().dual_evals++; }
    static void primary_ray() { op_counts().primary_rays++; }
    static void reflection_ray() { op_counts().reflection_rays++; }
    static void shadow_ray() { op_counts().shadow_rays++; }
    static void gi_ray() { op_counts().gi_rays++; }
    static int phase(int ph) {
        int prev = current_phase();
        current_phase() = ph;
        return prev;
    }
};

template <> struct Lit<CountF> { static CountF get(float f, double) { return CountF(f); } };

inline CountF o_sqrt(CountF x) { op_counts().sqrt++; return CountF(o_sqrt(x.v)); }
inline CountF o_sin(CountF x) { op_counts().trans++; return CountF(o_sin(x.v)); }
inline CountF o_cos(CountF x) { op_counts().trans++; return CountF(o_cos(x.v)); }
inline CountF o_tan(CountF x) { op_counts().trans++; return CountF(o_tan(x.v)); }
inline CountF o_exp(CountF x) { op_counts().trans++; return CountF(o_exp(x.v)); }
inline CountF o_pow(CountF x, CountF y) { op_counts().trans++; return CountF(o_pow(x.v, y.v)); }
inline CountF o_acos(CountF x) { op_counts().trans++; return CountF(o_acos(x.v)); }
inline CountF o_floor(CountF x) { op_counts().add++; return CountF(o_floor(x.v)); }
inline CountF o_round(CountF x) { op_counts().add++; return CountF(o_round(x.v)); }
inline CountF o_trunc(CountF x) { op_counts().add++; return CountF(o_trunc(x.v)); }
inline CountF o_abs(CountF x) { return CountF(o_abs(x.v)); }
inline CountF o_max(CountF a, CountF b) { op_counts().minmax++; return CountF(o_max(a.v, b.v)); }
inline CountF o_min(CountF a, CountF b) { op_counts().minmax++; return CountF(o_min(a.v, b.v)); }
inline bool o_isfinite(CountF x) { return o_isfinite(x.v); }
inline bool o_isnan(CountF x) { return o_isnan(x.v); }
inline double o_value(CountF x) { return x.v; }

}  // namespace oracle
