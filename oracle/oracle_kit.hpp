// oracle_kit.hpp — restatement of the MM3E kit (mm3e-kit/src) used by the render path.
//
// TEST INFRASTRUCTURE ONLY (parity checker + timed CPU baseline). Every function names the
// reference function it restates (path:line inside the MM3E repository) and keeps its
// floating-point operation order, so that the float instantiation reproduces the Rust f32
// results whenever the platform libm agrees.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle_math.hpp"

namespace oracle {

// ------------------------------------------------------------------------------------------
// vec.rs
// ------------------------------------------------------------------------------------------
template <class T> struct V3 {
    T x, y, z;
};
template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> splat(T v) { return V3<T>{v, v, v}; }
template <class T> inline V3<T> zero3() { return V3<T>{T(0), T(0), T(0)}; }
template <class T> inline V3<T> one3() { return V3<T>{T(1), T(1), T(1)}; }
// vec.rs:24-26  x*o.x + y*o.y + z*o.z
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vec.rs:27-29
template <class T> inline V3<T> cross(V3<T> a, V3<T> o) {
    return V3<T>{a.y * o.z - a.z * o.y, a.z * o.x - a.x * o.z, a.x * o.y - a.y * o.x};
}
template <class T> inline T length_sq(V3<T> a) { return dot(a, a); }
template <class T> inline T length(V3<T> a) { return o_sqrt(length_sq(a)); }
// vec.rs:45-47
template <class T> inline V3<T> scale(V3<T> a, T s) { return V3<T>{a.x * s, a.y * s, a.z * s}; }
// vec.rs:37-44  guarded against zero length
template <class T> inline V3<T> normalize(V3<T> a) {
    T len = length(a);
    if (len > OL(1e-12)) return scale(a, T(1) / len);
    return zero3<T>();
}
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return V3<T>{a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return V3<T>{a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return V3<T>{-a.x, -a.y, -a.z}; }
// vec.rs:49-51
template <class T> inline V3<T> cmul(V3<T> a, V3<T> o) { return V3<T>{a.x * o.x, a.y * o.y, a.z * o.z}; }
template <class T> inline V3<T> vabs(V3<T> a) { return V3<T>{o_abs(a.x), o_abs(a.y), o_abs(a.z)}; }
template <class T> inline V3<T> vmin(V3<T> a, V3<T> o) { return V3<T>{o_min(a.x, o.x), o_min(a.y, o.y), o_min(a.z, o.z)}; }
template <class T> inline V3<T> vmax(V3<T> a, V3<T> o) { return V3<T>{o_max(a.x, o.x), o_max(a.y, o.y), o_max(a.z, o.z)}; }
template <class T> inline V3<T> max_scalar(V3<T> a, T m) { return V3<T>{o_max(a.x, m), o_max(a.y, m), o_max(a.z, m)}; }
// vec.rs:64-66
template <class T> inline T max_element(V3<T> a) { return o_max(o_max(a.x, a.y), a.z); }
template <class T> inline V3<T> clamp01(V3<T> a) {
    return V3<T>{o_clamp(a.x, T(0), T(1)), o_clamp(a.y, T(0), T(1)), o_clamp(a.z, T(0), T(1))};
}
// vec.rs:71-73
template <class T> inline V3<T> clamp_to(V3<T> a, V3<T> lo, V3<T> hi) { return vmin(vmax(a, lo), hi); }
// vec.rs:75-77  self*(1-t) + o*t
template <class T> inline V3<T> mix(V3<T> a, V3<T> o, T t) { return scale(a, T(1) - t) + scale(o, t); }
// vec.rs:79-81
template <class T> inline V3<T> reflect(V3<T> a, V3<T> n) { return a - scale(n, T(2) * dot(a, n)); }
template <class T> inline bool is_zero(V3<T> a) { return a.x == T(0) && a.y == T(0) && a.z == T(0); }

// vec.rs:112-158 (columns)
template <class T> struct M3 {
    V3<T> c[3];
};
// vec.rs:125-127  cols[0]*v.x + cols[1]*v.y + cols[2]*v.z
template <class T> inline V3<T> mul_vec(const M3<T>& m, V3<T> v) {
    return scale(m.c[0], v.x) + scale(m.c[1], v.y) + scale(m.c[2], v.z);
}
// vec.rs:130-133
template <class T> inline M3<T> transpose(const M3<T>& m) {
    M3<T> r;
    r.c[0] = V3<T>{m.c[0].x, m.c[1].x, m.c[2].x};
    r.c[1] = V3<T>{m.c[0].y, m.c[1].y, m.c[2].y};
    r.c[2] = V3<T>{m.c[0].z, m.c[1].z, m.c[2].z};
    return r;
}

// vec.rs:165-222  rigid + uniform-scale transform
template <class T> struct Xform {
    M3<T> rot;
    V3<T> pos;
    T scale;
};
// vec.rs:190-192
template <class T> inline V3<T> to_world(const Xform<T>& x, V3<T> p) { return x.pos + mul_vec(x.rot, scale(p, x.scale)); }
// vec.rs:216-221
template <class T> inline V3<T> to_local(const Xform<T>& x, V3<T> p) {
    T inv = o_abs(x.scale) > OL(1e-12) ? T(1) / x.scale : T(0);
    return scale(mul_vec(transpose(x.rot), p - x.pos), inv);
}

// ------------------------------------------------------------------------------------------
// sdf.rs
// ------------------------------------------------------------------------------------------
template <class T> struct Field {
    T dist;
    uint32_t mat;
};
template <class T> inline Field<T> field_far() { return Field<T>{o_inf<T>(), 0u}; }

// sdf.rs:33-35
template <class T> inline T sd_sphere(V3<T> p, T r) { return length(p) - r; }
// sdf.rs:38-41
template <class T> inline T sd_box(V3<T> p, V3<T> half) {
    V3<T> q = vabs(p) - half;
    return length(max_scalar(q, T(0))) + o_min(max_element(q), T(0));
}
// sdf.rs:44-46
template <class T> inline T sd_round_box(V3<T> p, V3<T> half, T radius) { return sd_box(p, half - splat(radius)) - radius; }
// sdf.rs:49-51
template <class T> inline T sd_plane(V3<T> p, V3<T> n, T h) { return dot(p, n) + h; }
// sdf.rs:54-57
template <class T> inline T sd_torus(V3<T> p, T major, T minor) {
    T q = o_sqrt(p.x * p.x + p.z * p.z) - major;
    return o_sqrt(q * q + p.y * p.y) - minor;
}
// sdf.rs:60-66
template <class T> inline T sd_cylinder(V3<T> p, T h, T r) {
    T dx = o_sqrt(p.x * p.x + p.z * p.z) - r;
    T dy = o_abs(p.y) - h;
    T ox = o_max(dx, T(0));
    T oy = o_max(dy, T(0));
    return o_min(o_max(dx, dy), T(0)) + o_sqrt(ox * ox + oy * oy);
}
// sdf.rs:69-74
template <class T> inline T sd_capsule(V3<T> p, V3<T> a, V3<T> b, T r) {
    V3<T> pa = p - a;
    V3<T> ba = b - a;
    T h = o_clamp(dot(pa, ba) / dot(ba, ba), T(0), T(1));
    return length(pa - scale(ba, h)) - r;
}
// sdf.rs:78-91
template <class T> inline T sd_round_cone(V3<T> p, T r1, T r2, T h) {
    T qx = o_sqrt(p.x * p.x + p.z * p.z);
    T qy = p.y;
    T b = (r1 - r2) / o_max(h, OL(1e-6));
    T a = o_sqrt(o_max(T(1) - b * b, T(0)));
    T k = qx * -b + qy * a;
    if (k < T(0)) return o_sqrt(qx * qx + qy * qy) - r1;
    if (k > a * h) return o_sqrt(qx * qx + (qy - h) * (qy - h)) - r2;
    return qx * a + qy * b - r1;
}
// sdf.rs:94-101
template <class T> inline T sd_ellipsoid(V3<T> p, V3<T> r) {
    T k0 = length(V3<T>{p.x / r.x, p.y / r.y, p.z / r.z});
    if (k0 < OL(1e-6)) return -o_min(o_min(r.x, r.y), r.z);
    T k1 = length(V3<T>{p.x / (r.x * r.x), p.y / (r.y * r.y), p.z / (r.z * r.z)});
    return k0 * (k0 - T(1)) / o_max(k1, OL(1e-9));
}
// sdf.rs:104-107
template <class T> inline T sd_octahedron(V3<T> p, T s) {
    V3<T> q = vabs(p);
    return (q.x + q.y + q.z - s) * OL(0.5773503);
}
// sdf.rs:110-120
template <class T> inline T sd_hex_prism(V3<T> p, T r, T h) {
    const T kx = OL(-0.8660254), ky = OL(0.5), kz = OL(0.57735);
    V3<T> a = vabs(p);
    T t = T(2) * o_min(kx * a.x + ky * a.z, T(0));
    a.x = a.x - t * kx;
    a.z = a.z - t * ky;
    T clamped = o_clamp(a.x, -kz * r, kz * r);
    T dx = o_sqrt((a.x - clamped) * (a.x - clamped) + (a.z - r) * (a.z - r)) * o_signum(a.z - r);
    T dy = a.y - h;
    T mx = o_max(dx, T(0));
    T my = o_max(dy, T(0));
    return o_min(o_max(dx, dy), T(0)) + o_sqrt(mx * mx + my * my);
}

// sdf.rs:127-133
template <class T> inline Field<T> f_union(Field<T> a, Field<T> b) { return a.dist <= b.dist ? a : b; }
// sdf.rs:136-142
template <class T> inline Field<T> f_intersect(Field<T> a, Field<T> b) { return a.dist >= b.dist ? a : b; }
// sdf.rs:145-147
template <class T> inline Field<T> f_subtract(Field<T> a, Field<T> b) { return Field<T>{o_max(a.dist, -b.dist), a.mat}; }
// sdf.rs:152-160
template <class T> inline Field<T> f_smooth_union(Field<T> a, Field<T> b, T k) {
    if (k <= T(0)) return f_union(a, b);
    T h = o_clamp(OL(0.5) + OL(0.5) * (b.dist - a.dist) / k, T(0), T(1));
    T dist = b.dist * (T(1) - h) + a.dist * h - k * h * (T(1) - h);
    uint32_t mat = h > OL(0.5) ? a.mat : b.mat;
    return Field<T>{dist, mat};
}

// sdf.rs:192-236  domain operators
template <class T> inline T op_round(T d, T r) { return d - r; }
template <class T> inline T op_onion(T d, T t) { return o_abs(d) - t; }
template <class T> inline V3<T> op_elongate(V3<T> p, V3<T> h) { return p - clamp_to(p, scale(h, T(-1)), h); }
template <class T> inline T rep_axis(T v, T period) {
    if (period > T(0)) return v - period * o_round(v / period);
    return v;
}
template <class T> inline V3<T> op_repeat(V3<T> p, V3<T> period) {
    return V3<T>{rep_axis(p.x, period.x), rep_axis(p.y, period.y), rep_axis(p.z, period.z)};
}
template <class T> inline V3<T> op_twist(V3<T> p, T k) {
    T a = k * p.y;
    T s = o_sin(a), c = o_cos(a);
    return V3<T>{c * p.x - s * p.z, p.y, s * p.x + c * p.z};
}
template <class T> inline V3<T> op_bend(V3<T> p, T k) {
    T a = k * p.x;
    T s = o_sin(a), c = o_cos(a);
    return V3<T>{c * p.x - s * p.y, s * p.x + c * p.y, p.z};
}
template <class T> inline V3<T> op_mirror(V3<T> p, bool x, bool y, bool z) {
    return V3<T>{x ? o_abs(p.x) : p.x, y ? o_abs(p.y) : p.y, z ? o_abs(p.z) : p.z};
}

// ------------------------------------------------------------------------------------------
// dual.rs — forward-mode dual numbers (value + world-space gradient)
// ------------------------------------------------------------------------------------------
template <class T> struct Dual {
    T v;
    V3<T> g;
};
template <class T> inline Dual<T> dcon(T v) { return Dual<T>{v, zero3<T>()}; }
template <class T> inline Dual<T> dscale(Dual<T> a, T s) { return Dual<T>{a.v * s, scale(a.g, s)}; }  // dual.rs:30-32
template <class T> inline Dual<T> dadds(Dual<T> a, T s) { return Dual<T>{a.v + s, a.g}; }            // dual.rs:33-35
template <class T> inline Dual<T> dneg(Dual<T> a) { return Dual<T>{-a.v, -a.g}; }
template <class T> inline Dual<T> dabs(Dual<T> a) { return a.v >= T(0) ? a : dneg(a); }             // dual.rs:36-42
// dual.rs:43-47
template <class T> inline Dual<T> dsqrt(Dual<T> a) {
    T v = o_sqrt(o_max(a.v, T(0)));
    T k = v > OL(1e-9) ? OL(0.5) / v : T(0);
    return Dual<T>{v, scale(a.g, k)};
}
template <class T> inline Dual<T> dmin(Dual<T> a, Dual<T> o) { return a.v <= o.v ? a : o; }  // dual.rs:49-55
template <class T> inline Dual<T> dmax(Dual<T> a, Dual<T> o) { return a.v >= o.v ? a : o; }  // dual.rs:56-62
template <class T> inline Dual<T> dmax0(Dual<T> a) { return dmax(a, dcon(T(0))); }
template <class T> inline Dual<T> dmaxc(Dual<T> a, T c) { return a.v >= c ? a : dcon(c); }  // dual.rs:67-73
template <class T> inline Dual<T> dclamp(Dual<T> a, T lo, T hi) { return dmin(dmax(a, dcon(lo)), dcon(hi)); }
template <class T> inline Dual<T> dadd(Dual<T> a, Dual<T> o) { return Dual<T>{a.v + o.v, a.g + o.g}; }
template <class T> inline Dual<T> dsub(Dual<T> a, Dual<T> o) { return Dual<T>{a.v - o.v, a.g - o.g}; }
// dual.rs:98-103 product rule
template <class T> inline Dual<T> dmul(Dual<T> a, Dual<T> o) { return Dual<T>{a.v * o.v, scale(a.g, o.v) + scale(o.g, a.v)}; }
// dual.rs:106-112 quotient rule
template <class T> inline Dual<T> ddiv(Dual<T> a, Dual<T> o) {
    T inv2 = T(1) / (o.v * o.v);
    return Dual<T>{a.v / o.v, scale(scale(a.g, o.v) - scale(o.g, a.v), inv2)};
}

// dual.rs:129-131
template <class T> inline Dual<T> dd_sphere(Dual<T> x, Dual<T> y, Dual<T> z, T r) {
    return dadds(dsqrt(dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z))), -r);
}
// dual.rs:133-140
template <class T> inline Dual<T> dd_box(Dual<T> x, Dual<T> y, Dual<T> z, V3<T> half) {
    Dual<T> qx = dadds(dabs(x), -half.x), qy = dadds(dabs(y), -half.y), qz = dadds(dabs(z), -half.z);
    Dual<T> outside = dsqrt(dadd(dadd(dmul(dmax0(qx), dmax0(qx)), dmul(dmax0(qy), dmax0(qy))), dmul(dmax0(qz), dmax0(qz))));
    Dual<T> inside = dmin(dmax(qx, dmax(qy, qz)), dcon(T(0)));
    return dadd(outside, inside);
}
// dual.rs:142-144
template <class T> inline Dual<T> dd_round_box(Dual<T> x, Dual<T> y, Dual<T> z, V3<T> half, T radius) {
    return dadds(dd_box(x, y, z, half - splat(radius)), -radius);
}
// dual.rs:146-148
template <class T> inline Dual<T> dd_plane(Dual<T> x, Dual<T> y, Dual<T> z, V3<T> n, T h) {
    return dadds(dadd(dadd(dscale(x, n.x), dscale(y, n.y)), dscale(z, n.z)), h);
}
// dual.rs:150-153
template <class T> inline Dual<T> dd_torus(Dual<T> x, Dual<T> y, Dual<T> z, T major, T minor) {
    Dual<T> q = dadds(dsqrt(dadd(dmul(x, x), dmul(z, z))), -major);
    return dadds(dsqrt(dadd(dmul(q, q), dmul(y, y))), -minor);
}
// dual.rs:155-163
template <class T> inline Dual<T> dd_cylinder(Dual<T> x, Dual<T> y, Dual<T> z, T h, T r) {
    Dual<T> dx = dadds(dsqrt(dadd(dmul(x, x), dmul(z, z))), -r);
    Dual<T> dy = dadds(dabs(y), -h);
    Dual<T> inside = dmin(dmax(dx, dy), dcon(T(0)));
    Dual<T> ox = dmax0(dx), oy = dmax0(dy);
    return dadd(inside, dsqrt(dadd(dmul(ox, ox), dmul(oy, oy))));
}
// dual.rs:165-175
template <class T> inline Dual<T> dd_capsule(Dual<T> x, Dual<T> y, Dual<T> z, V3<T> a, V3<T> b, T r) {
    Dual<T> pax = dadds(x, -a.x), pay = dadds(y, -a.y), paz = dadds(z, -a.z);
    V3<T> ba = b - a;
    T dbb = o_max(dot(ba, ba), OL(1e-12));
    Dual<T> dpb = dadd(dadd(dscale(pax, ba.x), dscale(pay, ba.y)), dscale(paz, ba.z));
    Dual<T> hh = dclamp(dscale(dpb, T(1) / dbb), T(0), T(1));
    Dual<T> rx = dsub(pax, dscale(hh, ba.x)), ry = dsub(pay, dscale(hh, ba.y)), rz = dsub(paz, dscale(hh, ba.z));
    return dadds(dsqrt(dadd(dadd(dmul(rx, rx), dmul(ry, ry)), dmul(rz, rz))), -r);
}
// dual.rs:177-191
template <class T> inline Dual<T> dd_round_cone(Dual<T> x, Dual<T> y, Dual<T> z, T r1, T r2, T h) {
    Dual<T> qx = dsqrt(dadd(dmul(x, x), dmul(z, z)));
    Dual<T> qy = y;
    T b = (r1 - r2) / o_max(h, OL(1e-6));
    T a = o_sqrt(o_max(T(1) - b * b, T(0)));
    Dual<T> k = dadd(dscale(qx, -b), dscale(qy, a));
    if (k.v < T(0)) return dadds(dsqrt(dadd(dmul(qx, qx), dmul(qy, qy))), -r1);
    if (k.v > a * h) {
        Dual<T> qyh = dadds(qy, -h);
        return dadds(dsqrt(dadd(dmul(qx, qx), dmul(qyh, qyh))), -r2);
    }
    return dadds(dadd(dscale(qx, a), dscale(qy, b)), -r1);
}
// dual.rs:193-206
template <class T> inline Dual<T> dd_ellipsoid(Dual<T> x, Dual<T> y, Dual<T> z, V3<T> r) {
    Dual<T> k0x = dscale(x, T(1) / r.x), k0y = dscale(y, T(1) / r.y), k0z = dscale(z, T(1) / r.z);
    Dual<T> k0 = dsqrt(dadd(dadd(dmul(k0x, k0x), dmul(k0y, k0y)), dmul(k0z, k0z)));
    if (k0.v < OL(1e-6)) return dcon(-o_min(o_min(r.x, r.y), r.z));
    Dual<T> k1x = dscale(x, T(1) / (r.x * r.x)), k1y = dscale(y, T(1) / (r.y * r.y)), k1z = dscale(z, T(1) / (r.z * r.z));
    Dual<T> k1 = dmaxc(dsqrt(dadd(dadd(dmul(k1x, k1x), dmul(k1y, k1y)), dmul(k1z, k1z))), OL(1e-9));
    return ddiv(dmul(k0, dadds(k0, T(-1))), k1);
}
// dual.rs:208-210
template <class T> inline Dual<T> dd_octahedron(Dual<T> x, Dual<T> y, Dual<T> z, T s) {
    return dscale(dadds(dadd(dadd(dabs(x), dabs(y)), dabs(z)), -s), OL(0.5773503));
}
// dual.rs:212-232
template <class T> inline Dual<T> dd_hex_prism(Dual<T> x, Dual<T> y, Dual<T> z, T r, T h) {
    const T kx = OL(-0.8660254), ky = OL(0.5), kz = OL(0.57735);
    Dual<T> ax0 = dabs(x), az0 = dabs(z);
    Dual<T> ay = dadds(dabs(y), -h);
    Dual<T> tpre = dadd(dscale(ax0, kx), dscale(az0, ky));
    Dual<T> t = dscale(dmin(tpre, dcon(T(0))), T(2));
    Dual<T> ax = dsub(ax0, dscale(t, kx));
    Dual<T> az = dsub(az0, dscale(t, ky));
    Dual<T> clamped = dclamp(ax, -kz * r, kz * r);
    Dual<T> diffx = dsub(ax, clamped);
    Dual<T> diffz = dadds(az, -r);
    T sign = diffz.v >= T(0) ? T(1) : T(-1);
    Dual<T> dx = dscale(dsqrt(dadd(dmul(diffx, diffx), dmul(diffz, diffz))), sign);
    Dual<T> dy = ay;
    Dual<T> inside = dmin(dmax(dx, dy), dcon(T(0)));
    Dual<T> ox = dmax0(dx), oy = dmax0(dy);
    return dadd(inside, dsqrt(dadd(dmul(ox, ox), dmul(oy, oy))));
}
// dual.rs:246-251
template <class T> inline void dd_elongate(Dual<T>& x, Dual<T>& y, Dual<T>& z, V3<T> hg) {
    Dual<T> cx = dclamp(x, -hg.x, hg.x), cy = dclamp(y, -hg.y, hg.y), cz = dclamp(z, -hg.z, hg.z);
    x = dsub(x, cx);
    y = dsub(y, cy);
    z = dsub(z, cz);
}
// dual.rs:253-262
template <class T> inline Dual<T> dd_rep_axis(Dual<T> v, T period) {
    if (period > T(0)) return dadds(v, -o_round(v.v / period) * period);
    return v;
}
// dual.rs:278-291
template <class T> inline Dual<T> dd_union(Dual<T> a, Dual<T> b) { return dmin(a, b); }
template <class T> inline Dual<T> dd_subtract(Dual<T> a, Dual<T> b) { return dmax(a, dneg(b)); }
template <class T> inline Dual<T> dd_smooth_union(Dual<T> a, Dual<T> b, T k) {
    if (k <= T(0)) return dd_union(a, b);
    Dual<T> h = dclamp(dadds(dscale(dsub(b, a), OL(0.5) / k), OL(0.5)), T(0), T(1));
    Dual<T> omh = dsub(dcon(T(1)), h);
    return dsub(dadd(dmul(b, omh), dmul(a, h)), dscale(dmul(h, omh), k));
}

// ------------------------------------------------------------------------------------------
// volume.rs — sampled SDF grid
// ------------------------------------------------------------------------------------------
template <class T> struct Volume {
    uint64_t nx = 0, ny = 0, nz = 0;
    V3<T> min, cell;
    std::vector<T> data;
    // volume.rs:91-94
    T at(uint64_t i, uint64_t j, uint64_t k) const { return data[(k * ny + j) * nx + i]; }
    // volume.rs:47-62
    bool has_valid_layout() const {
        return nx >= 2 && ny >= 2 && nz >= 2 && o_isfinite(min.x) && o_isfinite(min.y) && o_isfinite(min.z) &&
               o_isfinite(cell.x) && o_isfinite(cell.y) && o_isfinite(cell.z) && cell.x > T(0) && cell.y > T(0) &&
               cell.z > T(0) && data.size() == nx * ny * nz;
    }
    // volume.rs:97-103
    void bounds(V3<T>& lo, V3<T>& hi) const {
        T sx = T((float)(nx - 1)) * cell.x;
        T sy = T((float)(ny - 1)) * cell.y;
        T sz = T((float)(nz - 1)) * cell.z;
        lo = min;
        hi = min + V3<T>{sx, sy, sz};
    }
    // volume.rs:106-113
    T max_cell() const { return o_max(o_max(cell.x, cell.y), cell.z); }
    T recommended_normal_h() const { return max_cell() * OL(0.6); }
    // volume.rs:194-228
    T sample(V3<T> p) const {
        if (!has_valid_layout()) return o_inf<T>();
        V3<T> lo, hi;
        bounds(lo, hi);
        V3<T> c = clamp_to(p, lo, hi);
        T outside = length(p - c);
        V3<T> g{(c.x - min.x) / cell.x, (c.y - min.y) / cell.y, (c.z - min.z) / cell.z};
        auto clampi = [](T v, uint64_t n) {
            uint64_t i = o_to_usize(o_max(o_floor(v), T(0)));
            return i < n - 2 ? i : n - 2;
        };
        uint64_t i0 = clampi(g.x, nx), j0 = clampi(g.y, ny), k0 = clampi(g.z, nz);
        T fx = o_clamp(g.x - T((float)i0), T(0), T(1));
        T fy = o_clamp(g.y - T((float)j0), T(0), T(1));
        T fz = o_clamp(g.z - T((float)k0), T(0), T(1));
        auto lerp = [](T a, T b, T t) { return a + (b - a) * t; };
        T x00 = lerp(at(i0, j0, k0), at(i0 + 1, j0, k0), fx);
        T x10 = lerp(at(i0, j0 + 1, k0), at(i0 + 1, j0 + 1, k0), fx);
        T x01 = lerp(at(i0, j0, k0 + 1), at(i0 + 1, j0, k0 + 1), fx);
        T x11 = lerp(at(i0, j0 + 1, k0 + 1), at(i0 + 1, j0 + 1, k0 + 1), fx);
        T d = lerp(lerp(x00, x10, fy), lerp(x01, x11, fy), fz);
        if (!o_isfinite(d)) return o_inf<T>();
        if (outside > T(0)) return o_max(outside, d - outside);
        return d;
    }
};

// ------------------------------------------------------------------------------------------
// csg.rs — object-local expression trees (node array, children by index)
// ------------------------------------------------------------------------------------------
enum {
    K_SPHERE = 0, K_BOX, K_ROUND_BOX, K_TORUS, K_CYLINDER, K_CAPSULE, K_CONE, K_ELLIPSOID,
    K_OCTAHEDRON, K_HEX_PRISM, K_PLANE, K_CSG, K_VOLUME, K_SURFACE
};
enum { C_TRANSFORM = 100, C_UNION, C_INTERSECT, C_SUBTRACT, C_SMOOTH_UNION, C_OFFSET, C_SHELL };

template <class T> struct CsgNode {
    uint32_t kind, a, b;
    T p[7];
    Xform<T> xf;
};

// Analytic primitive distance by kind (Prim::distance, mm3e-orchestrator/src/lib.rs:215-233;
// csg.rs:97-107).
template <class T> inline T prim_distance(uint32_t kind, const T* q, V3<T> l) {
    switch (kind) {
        case K_SPHERE: return sd_sphere(l, q[0]);
        case K_BOX: return sd_box(l, V3<T>{q[0], q[1], q[2]});
        case K_ROUND_BOX: return sd_round_box(l, V3<T>{q[0], q[1], q[2]}, q[3]);
        case K_TORUS: return sd_torus(l, q[0], q[1]);
        case K_CYLINDER: return sd_cylinder(l, q[0], q[1]);
        case K_CAPSULE: return sd_capsule(l, V3<T>{q[0], q[1], q[2]}, V3<T>{q[3], q[4], q[5]}, q[6]);
        case K_CONE: return sd_round_cone(l, q[0], q[1], q[2]);
        case K_ELLIPSOID: return sd_ellipsoid(l, V3<T>{q[0], q[1], q[2]});
        case K_OCTAHEDRON: return sd_octahedron(l, q[0]);
        case K_HEX_PRISM: return sd_hex_prism(l, q[0], q[1]);
        case K_PLANE: return sd_plane(l, V3<T>{q[0], q[1], q[2]}, q[3]);
        default: return o_inf<T>();
    }
}

// csg.rs:95-118
template <class T> inline T csg_distance(const std::vector<CsgNode<T>>& nodes, uint32_t i, V3<T> p) {
    const CsgNode<T>& n = nodes[i];
    switch (n.kind) {
        case C_TRANSFORM: return csg_distance(nodes, n.a, to_local(n.xf, p)) * n.xf.scale;
        case C_UNION: return o_min(csg_distance(nodes, n.a, p), csg_distance(nodes, n.b, p));
        case C_INTERSECT: return o_max(csg_distance(nodes, n.a, p), csg_distance(nodes, n.b, p));
        case C_SUBTRACT: return o_max(csg_distance(nodes, n.a, p), -csg_distance(nodes, n.b, p));
        case C_SMOOTH_UNION: {
            T da = csg_distance(nodes, n.a, p);
            T db = csg_distance(nodes, n.b, p);
            return f_smooth_union(Field<T>{da, 0}, Field<T>{db, 0}, n.p[0]).dist;
        }
        case C_OFFSET: return csg_distance(nodes, n.a, p) - n.p[0];
        case C_SHELL: return o_abs(csg_distance(nodes, n.a, p)) - n.p[0];
        default: return prim_distance(n.kind, n.p, p);
    }
}

// csg.rs:86-97
template <class T> inline void csg_enclose(V3<T> a, T ar, V3<T> b, T br, V3<T>& c, T& r) {
    V3<T> delta = b - a;
    T d = length(delta);
    if (d + br <= ar) { c = a; r = ar; return; }
    if (d + ar <= br) { c = b; r = br; return; }
    r = (d + ar + br) * OL(0.5);
    c = a + scale(delta, (r - ar) / o_max(d, OL(1e-12)));
}

// csg.rs:120-150  returns false for "None"
template <class T> inline bool csg_bound(const std::vector<CsgNode<T>>& nodes, uint32_t i, V3<T>& c, T& r) {
    const CsgNode<T>& n = nodes[i];
    const T* q = n.p;
    switch (n.kind) {
        case K_SPHERE: c = zero3<T>(); r = q[0]; return true;
        case K_BOX: case K_ROUND_BOX: c = zero3<T>(); r = length(V3<T>{q[0], q[1], q[2]}); return true;
        case K_TORUS: c = zero3<T>(); r = q[0] + q[1]; return true;
        case K_CYLINDER: c = zero3<T>(); r = o_sqrt(q[0] * q[0] + q[1] * q[1]); return true;
        case K_CAPSULE: {
            V3<T> a{q[0], q[1], q[2]}, b{q[3], q[4], q[5]};
            c = scale(a + b, OL(0.5));
            r = length(a - b) * OL(0.5) + q[6];
            return true;
        }
        case K_CONE: c = V3<T>{T(0), q[2] * OL(0.5), T(0)}; r = q[2] * OL(0.5) + o_max(q[0], q[1]); return true;
        case K_ELLIPSOID: case K_OCTAHEDRON: case K_PLANE: return false;
        case K_HEX_PRISM: c = zero3<T>(); r = o_sqrt(T(4) * q[0] * q[0] / T(3) + q[1] * q[1]); return true;
        case C_TRANSFORM: {
            V3<T> cc; T rr;
            if (!csg_bound(nodes, n.a, cc, rr)) return false;
            c = to_world(n.xf, cc);
            r = rr * n.xf.scale;
            return true;
        }
        case C_UNION: case C_SMOOTH_UNION: {
            V3<T> ac, bc; T ar, br;
            if (!csg_bound(nodes, n.a, ac, ar)) return false;
            if (!csg_bound(nodes, n.b, bc, br)) return false;
            csg_enclose(ac, ar, bc, br, c, r);
            if (n.kind == C_SMOOTH_UNION) r = r + n.p[0] * OL(0.25);
            return true;
        }
        case C_INTERSECT: {
            V3<T> ac, bc; T ar, br;
            bool ha = csg_bound(nodes, n.a, ac, ar);
            bool hb = csg_bound(nodes, n.b, bc, br);
            if (ha && hb) {
                if (ar <= br) { c = ac; r = ar; } else { c = bc; r = br; }
                return true;
            }
            if (ha) { c = ac; r = ar; return true; }
            if (hb) { c = bc; r = br; return true; }
            return false;
        }
        case C_SUBTRACT: return csg_bound(nodes, n.a, c, r);
        case C_OFFSET: {
            if (!csg_bound(nodes, n.a, c, r)) return false;
            r = o_max(r + n.p[0], T(0));
            return true;
        }
        case C_SHELL: {
            if (!csg_bound(nodes, n.a, c, r)) return false;
            r = r + n.p[0];
            return true;
        }
        default: return false;
    }
}

// ------------------------------------------------------------------------------------------
// camera.rs
// ------------------------------------------------------------------------------------------
template <class T> struct Ray {
    V3<T> origin, dir;
};
// march.rs:21-23
template <class T> inline V3<T> ray_at(const Ray<T>& r, T t) { return r.origin + scale(r.dir, t); }

template <class T> struct Camera {
    V3<T> eye, forward, right, up;
    T fov_scale;
};
// camera.rs:50-55
template <class T> inline Camera<T> camera_look_at(V3<T> eye, V3<T> target, V3<T> up_hint, T fov_y) {
    Camera<T> c;
    c.eye = eye;
    c.forward = normalize(target - eye);
    c.right = normalize(cross(c.forward, up_hint));
    c.up = cross(c.right, c.forward);
    c.fov_scale = o_tan(fov_y * OL(0.5));
    return c;
}
// camera.rs:59-65
template <class T> inline Ray<T> camera_ray(const Camera<T>& c, T sx, T sy, uint32_t w, uint32_t h) {
    T wf = T((float)w), hf = T((float)h);
    T aspect = wf / hf;
    T ndc_x = (T(2) * sx / wf - T(1)) * aspect * c.fov_scale;
    T ndc_y = (T(1) - T(2) * sy / hf) * c.fov_scale;
    V3<T> dir = normalize(c.forward + scale(c.right, ndc_x) + scale(c.up, ndc_y));
    return Ray<T>{c.eye, dir};
}

// ------------------------------------------------------------------------------------------
// march.rs — Marcher
// ------------------------------------------------------------------------------------------
template <class T> struct Hit {
    bool hit;
    T t;
    V3<T> pos, normal;
    uint32_t mat, steps;
};

template <class T> struct Marcher {
    uint32_t max_steps = 160;
    T max_dist = T(120);
    T eps = OL(0.0006);
    T step_scale = T(1);
    uint32_t shadow_steps = 64;
    uint32_t ao_samples = 5;
    T lod_footprint = T(0);
    T subitize = T(0);
    bool secant = false;
    T normal_h = OL(0.0009);

    // march.rs:120-209  enhanced sphere tracing with overlap-failure rollback
    template <class F, class N> Hit<T> march_with(const F& field, const N& normal_fn, const Ray<T>& ray) const {
        enum { OMEGA, LEAP, SECANT };
        T omega = step_scale >= T(1) ? OL(1.4) : step_scale;
        T sub = step_scale >= T(1) ? subitize : T(0);
        bool secant_on = secant && step_scale >= T(1);
        int boost = OMEGA;
        T t = T(0), prev_radius = T(0), step_len = T(0), t_prev = T(0);
        T d_prev = o_inf<T>();
        for (uint32_t i = 0; i < max_steps; ++i) {
            V3<T> p = ray_at(ray, t);
            Field<T> f = field(p);
            T radius = o_abs(f.dist);
            T e = eps * (T(1) + t * OL(0.5)) + lod_footprint * t;
            if ((step_len > T(0) && f.dist < T(0)) || step_len > radius + prev_radius) {
                T gap_lo = t_prev + prev_radius;
                T gap_hi = t - radius;
                T mid = OL(0.5) * (gap_lo + gap_hi);
                bool covered = f.dist > T(0) && field(ray_at(ray, mid)).dist >= OL(0.5) * (gap_hi - gap_lo);
                if (!covered) {
                    t = gap_lo;
                    if (boost == OMEGA) omega = o_min(omega, T(1));
                    else if (boost == LEAP) sub = T(0);
                    else secant_on = false;
                    boost = OMEGA;
                    prev_radius = T(0);
                    step_len = T(0);
                    d_prev = o_inf<T>();
                    continue;
                }
            }
            if (f.dist < e) return Hit<T>{true, t, p, normal_fn(p), f.mat, i};
            step_len = f.dist * omega;
            boost = OMEGA;
            if (sub > T(0) && f.dist > e * T(6)) {
                step_len = step_len * (T(1) + sub);
                boost = LEAP;
            }
            if (secant_on && f.dist < OL(0.08) && o_isfinite(d_prev)) {
                T dt = t - t_prev;
                T dd = f.dist - d_prev;
                if (dt > OL(1e-6) && dd < -OL(1e-6)) {
                    step_len = o_clamp(-f.dist * dt / dd, f.dist, f.dist * T(4));
                    boost = SECANT;
                }
            }
            prev_radius = radius;
            d_prev = f.dist;
            t_prev = t;
            t = t + step_len;
            if (t > max_dist) break;
        }
        return Hit<T>{false, t, ray_at(ray, t), zero3<T>(), 0u, max_steps};
    }

    // march.rs:212-223  tetrahedron normal
    template <class F> V3<T> normal(const F& field, V3<T> p) const {
        T h = normal_h;
        V3<T> k0{T(1), T(-1), T(-1)}, k1{T(-1), T(-1), T(1)}, k2{T(-1), T(1), T(-1)}, k3{T(1), T(1), T(1)};
        V3<T> g = scale(k0, field(p + scale(k0, h)).dist) + scale(k1, field(p + scale(k1, h)).dist) +
                  scale(k2, field(p + scale(k2, h)).dist) + scale(k3, field(p + scale(k3, h)).dist);
        return normalize(g);
    }

    // march.rs:227-259  jittered soft shadow
    template <class F> T soft_shadow(const F& field, V3<T> origin, V3<T> dir, T max_t, T k) const {
        T res = T(1);
        T hb = origin.x * OL(127.1) + origin.y * OL(311.7) + origin.z * OL(74.7);
        T jitter = o_abs(o_fract(o_sin(hb) * OL(43758.547)));
        T t = OL(0.02) + jitter * OL(0.16);
        for (uint32_t s = 0; s < shadow_steps; ++s) {
            T h = field(origin + scale(dir, t)).dist;
            if (h < OL(0.0008)) return T(0);
            res = o_min(res, k * h / t);
            t = t + o_clamp(h, OL(0.06), OL(0.5) + OL(0.7) * t);
            if (t > max_t) break;
        }
        return o_clamp(res, T(0), T(1));
    }

    // march.rs:264-280
    template <class F> T ambient_occlusion(const F& field, V3<T> p, V3<T> n) const {
        uint32_t ns = ao_samples;
        if (ns == 0) return T(1);
        T base = o_max(normal_h, OL(0.01));
        T span = T((float)((ns > 2 ? ns : 2) - 1));
        T occ = T(0), sca = T(1);
        for (uint32_t i = 0; i < ns; ++i) {
            T hr = base + OL(0.12) * T((float)i) / span;
            T d = field(p + scale(n, hr)).dist;
            occ = occ + (hr - d) * sca;
            sca = sca * OL(0.92);
        }
        return o_clamp(T(1) - OL(2.6) * occ, T(0), T(1));
    }
};

// ------------------------------------------------------------------------------------------
// shade.rs
// ------------------------------------------------------------------------------------------
template <class T> inline T pi_f() { return OL(3.14159265358979323846); }
template <class T> inline T lambert(V3<T> n, V3<T> l) { return o_max(dot(n, l), T(0)); }  // shade.rs:9-11
// shade.rs:14-17
template <class T> inline T fresnel_schlick(T cos_theta, T f0) {
    T m = o_clamp(T(1) - cos_theta, T(0), T(1));
    return f0 + (T(1) - f0) * o_powi5(m);
}
// shade.rs:20-23
template <class T> inline V3<T> fresnel_schlick_vec(T cos_theta, V3<T> f0) {
    T m = o_powi5(o_clamp(T(1) - cos_theta, T(0), T(1)));
    return f0 + scale(one3<T>() - f0, m);
}
// shade.rs:26-28
template <class T> inline T luminance(V3<T> c) { return c.x * OL(0.2126) + c.y * OL(0.7152) + c.z * OL(0.0722); }
// shade.rs:31-36
template <class T> inline T d_ggx(T noh, T a2) {
    T d = noh * noh * (a2 - T(1)) + T(1);
    return a2 / o_max(pi_f<T>() * d * d, OL(1e-12));
}
// shade.rs:39-43
template <class T> inline T v_smith(T nol, T nov, T a2) {
    T gv = nol * o_sqrt(nov * nov * (T(1) - a2) + a2);
    T gl = nov * o_sqrt(nol * nol * (T(1) - a2) + a2);
    return OL(0.5) / o_max(gv + gl, OL(1e-5));
}
// shade.rs:51-72
template <class T>
inline V3<T> brdf(V3<T> n, V3<T> l, V3<T> view, V3<T> albedo, T metallic, T roughness, T reflectance) {
    T nol = o_max(dot(n, l), T(0));
    if (nol <= T(0)) return zero3<T>();
    T nov = o_max(dot(n, view), OL(1e-4));
    V3<T> h = normalize(l + view);
    T noh = o_max(dot(n, h), T(0));
    T voh = o_max(dot(view, h), T(0));
    T a = o_max(roughness * roughness, OL(1e-3));
    T a2 = a * a;
    V3<T> f0 = mix(splat(OL(0.08) * o_clamp(reflectance, T(0), T(1))), albedo, metallic);
    V3<T> f = fresnel_schlick_vec(voh, f0);
    V3<T> spec = scale(f, d_ggx(noh, a2) * v_smith(nol, nov, a2));
    V3<T> kd = scale(one3<T>() - f, T(1) - metallic);
    V3<T> diff = scale(cmul(kd, albedo), T(1) / pi_f<T>());
    return scale(diff + spec, nol);
}
// shade.rs:76-84
template <class T> inline V3<T> sky(V3<T> dir, V3<T> sun_dir) {
    T t = o_clamp(OL(0.5) * (dir.y + T(1)), T(0), T(1));
    V3<T> horizon{OL(0.78), OL(0.86), OL(0.96)};
    V3<T> zenith{OL(0.20), OL(0.38), OL(0.72)};
    V3<T> base = mix(horizon, zenith, t);
    T sun = o_max(dot(dir, sun_dir), T(0));
    T glow = o_pow(sun, T(8)) * OL(0.3) + o_pow(sun, T(220)) * T(6);
    return base + splat(glow);
}
// shade.rs:88-95
template <class T> inline V3<T> sky_diffuse(V3<T> dir, V3<T> sun_dir) {
    T t = o_clamp(OL(0.5) * (dir.y + T(1)), T(0), T(1));
    V3<T> horizon{OL(0.78), OL(0.86), OL(0.96)};
    V3<T> zenith{OL(0.20), OL(0.38), OL(0.72)};
    V3<T> base = mix(horizon, zenith, t);
    T soft = o_pow(o_max(dot(dir, sun_dir), T(0)), T(8)) * OL(0.3);
    return base + splat(soft);
}
// shade.rs:98-104
template <class T> inline T aces1(T v) {
    v = o_max(v, T(0));
    return o_clamp((v * (OL(2.51) * v + OL(0.03))) / (v * (OL(2.43) * v + OL(0.59)) + OL(0.14)), T(0), T(1));
}
template <class T> inline V3<T> aces(V3<T> x) { return V3<T>{aces1(x.x), aces1(x.y), aces1(x.z)}; }
// shade.rs:107-110
template <class T> inline V3<T> gamma(V3<T> x) {
    T inv = T(1) / OL(2.2);
    return V3<T>{o_pow(o_max(x.x, T(0)), inv), o_pow(o_max(x.y, T(0)), inv), o_pow(o_max(x.z, T(0)), inv)};
}
// shade.rs:113-116
template <class T> inline V3<T> apply_fog(V3<T> color, V3<T> fog, T t, T density) {
    T f = T(1) - o_exp(-t * density);
    return mix(color, fog, o_clamp(f, T(0), T(1)));
}

// ------------------------------------------------------------------------------------------
// lib.rs atoms — FNV-1a hash (mm3e-kit/src/lib.rs:63-78)
// ------------------------------------------------------------------------------------------
inline uint64_t fnv1a(const uint8_t* bytes, size_t n) {
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= (uint64_t)bytes[i];
        h *= 0x00000100000001b3ull;
    }
    return h;
}
inline float hash_cell(int32_t ix, int32_t iy) {
    uint8_t buf[8];
    uint32_t ux = (uint32_t)ix, uy = (uint32_t)iy;
    for (int i = 0; i < 4; ++i) {
        buf[i] = (uint8_t)(ux >> (8 * i));
        buf[4 + i] = (uint8_t)(uy >> (8 * i));
    }
    return (float)(fnv1a(buf, 8) >> 40) / (float)(1ull << 24);
}

}  // namespace oracle
