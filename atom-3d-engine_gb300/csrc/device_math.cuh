// device_math.cuh — binary32 vector math, SDF primitives, CSG programs and the world field
// interpreter for the MM3E scene tape (device side).
//
// Every formula restates the reference function cited beside it and keeps its operation
// order; scalar semantics follow Rust f32 (fmaxf/fminf ignore NaN, clamp is two compares,
// signum(+-0) = +-1, round is half-away-from-zero).
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "tape.h"

namespace mm3e {

#define MD __device__ __forceinline__

struct V {
    float x, y, z;
};
MD V mk(float x, float y, float z) { return V{x, y, z}; }
MD V splat(float v) { return V{v, v, v}; }
MD V operator+(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
MD V operator-(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
MD V operator-(V a) { return V{-a.x, -a.y, -a.z}; }
MD V scale(V a, float s) { return V{a.x * s, a.y * s, a.z * s}; }
MD V cmul(V a, V b) { return V{a.x * b.x, a.y * b.y, a.z * b.z}; }
MD float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }  // vec.rs:24-26
MD V cross(V a, V o) { return V{a.y * o.z - a.z * o.y, a.z * o.x - a.x * o.z, a.x * o.y - a.y * o.x}; }
MD float length_sq(V a) { return dot(a, a); }
MD float length(V a) { return sqrtf(length_sq(a)); }
MD V normalize(V a) {  // vec.rs:37-44
    float len = length(a);
    if (len > 1e-12f) return scale(a, 1.0f / len);
    return V{0.0f, 0.0f, 0.0f};
}
MD V vabs(V a) { return V{fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
MD V vmin(V a, V b) { return V{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
MD V vmax(V a, V b) { return V{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
MD V max_scalar(V a, float m) { return V{fmaxf(a.x, m), fmaxf(a.y, m), fmaxf(a.z, m)}; }
MD float max_element(V a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
MD float clampf(float x, float lo, float hi) {  // core::f32::clamp
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
MD V clamp01(V a) { return V{clampf(a.x, 0.f, 1.f), clampf(a.y, 0.f, 1.f), clampf(a.z, 0.f, 1.f)}; }
MD V mix(V a, V o, float t) { return scale(a, 1.0f - t) + scale(o, t); }  // vec.rs:75-77
MD V reflect(V a, V n) { return a - scale(n, 2.0f * dot(a, n)); }       // vec.rs:79-81
MD V ld3(const float* p) { return V{p[0], p[1], p[2]}; }
MD bool is_zero(V a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
MD float signum(float x) {
    if (x != x) return x;
    return signbit(x) ? -1.0f : 1.0f;
}
MD float powi5(float x) {  // LLVM powi(x, 5) expansion
    float x2 = x * x;
    float x4 = x2 * x2;
    return x * x4;
}
// R columns c0..c2: R^T v = (dot(c0,v), dot(c1,v), dot(c2,v)) (vec.rs:125-133, 216-221)
MD V rot_t(const float* r, V v) {
    return V{r[0] * v.x + r[1] * v.y + r[2] * v.z, r[3] * v.x + r[4] * v.y + r[5] * v.z,
             r[6] * v.x + r[7] * v.y + r[8] * v.z};
}
// rot_t for r exactly the identity, with the same result bits for finite v. There x is
// (1·vx + 0·vy) + 0·vz: the products 0·vy and 0·vz are zeros carrying the signs of vy and vz,
// so x is vx except for the sign of a zero vx, which IEEE zero addition leaves negative only when
// vy and vz are negative too. Adding the zero whose sign is that AND of signs reproduces it (and
// likewise for y and z), one integer and one float operation a component instead of four.
MD float zero_with_sign_and(float a, float b) {
    return __int_as_float((__float_as_int(a) & __float_as_int(b)) & (int)0x80000000u);
}
MD V rot_t_identity(V v) {
    return V{v.x + zero_with_sign_and(v.y, v.z), v.y + zero_with_sign_and(v.x, v.z), v.z + zero_with_sign_and(v.x, v.y)};
}

struct Field {
    float d;
    uint32_t m;
};

// ---- sdf.rs primitives (local space) ----
MD float sd_sphere(V p, float r) { return length(p) - r; }
MD float sd_box(V p, V half) {
    V q = vabs(p) - half;
    return length(max_scalar(q, 0.0f)) + fminf(max_element(q), 0.0f);
}
MD float sd_torus(V p, float major, float minor) {
    float q = sqrtf(p.x * p.x + p.z * p.z) - major;
    return sqrtf(q * q + p.y * p.y) - minor;
}
MD float sd_cylinder(V p, float h, float r) {
    float dx = sqrtf(p.x * p.x + p.z * p.z) - r;
    float dy = fabsf(p.y) - h;
    float ox = fmaxf(dx, 0.0f), oy = fmaxf(dy, 0.0f);
    return fminf(fmaxf(dx, dy), 0.0f) + sqrtf(ox * ox + oy * oy);
}
MD float sd_capsule(V p, V a, V b, float r) {
    V pa = p - a, ba = b - a;
    float h = clampf(dot(pa, ba) / dot(ba, ba), 0.0f, 1.0f);
    return length(pa - scale(ba, h)) - r;
}
MD float sd_round_cone(V p, float r1, float r2, float h) {
    float qx = sqrtf(p.x * p.x + p.z * p.z), qy = p.y;
    float b = (r1 - r2) / fmaxf(h, 1e-6f);
    float a = sqrtf(fmaxf(1.0f - b * b, 0.0f));
    float k = qx * -b + qy * a;
    if (k < 0.0f) return sqrtf(qx * qx + qy * qy) - r1;
    if (k > a * h) return sqrtf(qx * qx + (qy - h) * (qy - h)) - r2;
    return qx * a + qy * b - r1;
}
MD float sd_ellipsoid(V p, V r) {
    float k0 = length(V{p.x / r.x, p.y / r.y, p.z / r.z});
    if (k0 < 1e-6f) return -fminf(fminf(r.x, r.y), r.z);
    float k1 = length(V{p.x / (r.x * r.x), p.y / (r.y * r.y), p.z / (r.z * r.z)});
    return k0 * (k0 - 1.0f) / fmaxf(k1, 1e-9f);
}
MD float sd_octahedron(V p, float s) {
    V q = vabs(p);
    return (q.x + q.y + q.z - s) * 0.5773503f;
}
MD float sd_hex_prism(V p, float r, float h) {
    const float kx = -0.8660254f, ky = 0.5f, kz = 0.57735f;
    V a = vabs(p);
    float t = 2.0f * fminf(kx * a.x + ky * a.z, 0.0f);
    a.x = a.x - t * kx;
    a.z = a.z - t * ky;
    float cl = clampf(a.x, -kz * r, kz * r);
    float dx = sqrtf((a.x - cl) * (a.x - cl) + (a.z - r) * (a.z - r)) * signum(a.z - r);
    float dy = a.y - h;
    float mx = fmaxf(dx, 0.0f), my = fmaxf(dy, 0.0f);
    return fminf(fmaxf(dx, dy), 0.0f) + sqrtf(mx * mx + my * my);
}
// Prim::distance for the 11 analytic kinds (lib.rs:215-233)
MD float prim_distance(uint32_t kind, const float* q, V l) {
    switch (kind) {
        case 0: return sd_sphere(l, q[0]);
        case 1: return sd_box(l, V{q[0], q[1], q[2]});
        case 2: return sd_box(l, V{q[0], q[1], q[2]} - splat(q[3])) - q[3];
        case 3: return sd_torus(l, q[0], q[1]);
        case 4: return sd_cylinder(l, q[0], q[1]);
        case 5: return sd_capsule(l, V{q[0], q[1], q[2]}, V{q[3], q[4], q[5]}, q[6]);
        case 6: return sd_round_cone(l, q[0], q[1], q[2]);
        case 7: return sd_ellipsoid(l, V{q[0], q[1], q[2]});
        case 8: return sd_octahedron(l, q[0]);
        case 9: return sd_hex_prism(l, q[0], q[1]);
        case 10: return dot(l, V{q[0], q[1], q[2]}) + q[3];
        default: return __int_as_float(0x7f800000);
    }
}

// ---- sdf.rs combinators ----
MD Field f_union(Field a, Field b) { return a.d <= b.d ? a : b; }
MD Field f_subtract(Field a, Field b) { return Field{fmaxf(a.d, -b.d), a.m}; }
MD Field f_smooth_union(Field a, Field b, float k) {  // sdf.rs:152-160
    if (k <= 0.0f) return f_union(a, b);
    float h = clampf(0.5f + 0.5f * (b.d - a.d) / k, 0.0f, 1.0f);
    float dist = b.d * (1.0f - h) + a.d * h - k * h * (1.0f - h);
    return Field{dist, h > 0.5f ? a.m : b.m};
}
MD float rep_axis(float v, float period) { return period > 0.0f ? v - period * roundf(v / period) : v; }

// Squared norms for the cull pre-tests below, with fused multiply-adds: within a few units of
// roundoff of length_sq (both are within three of the exact square of the same binary32
// vector), which the tests' margins absorb. Never a value that the field returns.
MD float length_sq_fma(V a) { return __fmaf_rn(a.x, a.x, __fmaf_rn(a.y, a.y, a.z * a.z)); }
MD V rot_t_fma(const float* r, V v) {
    return V{__fmaf_rn(r[0], v.x, __fmaf_rn(r[1], v.y, r[2] * v.z)), __fmaf_rn(r[3], v.x, __fmaf_rn(r[4], v.y, r[5] * v.z)),
             __fmaf_rn(r[6], v.x, __fmaf_rn(r[7], v.y, r[8] * v.z))};
}

// Cull pre-test of a bounded union member (accel.rs:98-100: a sphere whose lower bound exceeds the
// best distance so far cannot win). With d2 the squared distance |p - c|^2 (length_sq, as length()
// computes it, or length_sq_fma), true only when fl(fl(sqrt(length_sq(p - c))) - r) > bd holds
// for certain: squared distances with a relative margin of 2^-14, far wider than the few
// roundings on either side, and only for bd >= 0 (where a margin proportional to bd + r also
// clears bd's own rounding step). Skips the square root of members that the exact test would
// cull anyway; never culls one that it would keep.
MD bool far_beyond(float d2, float bd, float r) {
    float q = bd + r;
    return bd >= 0.0f && d2 > q * q * 1.00006103515625f;
}
// Linearised pre-tests. cull_base(p) = fl(|p|^2 mu), mu = 1 - 2^-19, once per field evaluation;
// dist2_below(p, base, -2c, mu |c|^2 rounded down) = fl((base + c2) - 2 p.c) in fused
// multiply-adds. Its roundings stay within 11 units of roundoff (2^-24 each) of |p|^2 + |c|^2,
// less than the 2^-19 (|p|^2 + |c|^2) that mu takes off, so it never exceeds |p - c|^2.
// far_beyond_lin(d2, bd, 2 M r, M r^2) with M = 1 + 2^-14 and both constants rounded up: d2 above
// fl(M bd^2 + 2 M r bd + M r^2) puts |p - c|^2 above (bd + r)^2 (1 + 2^-15), and from there
// fl(fl(sqrt(length_sq(p - c))) - r) > bd for bd >= 0 as in far_beyond. Three fused
// multiply-adds and one addition for the distance, two for the threshold: fewer instructions than
// the difference vector, its norm and the squared threshold.
MD float cull_base(V p) { return length_sq_fma(p) * 0.99999809265136719f; }
MD float dist2_below(V p, float base, float ax, float ay, float az, float c2) {
    return __fmaf_rn(p.x, ax, __fmaf_rn(p.y, ay, __fmaf_rn(p.z, az, base + c2)));
}
MD bool far_beyond_lin(float d2, float bd, float m2r, float mr2) {
    return bd >= 0.0f && d2 > __fmaf_rn(bd, __fmaf_rn(bd, 1.00006103515625f, m2r), mr2);
}
MD bool far_beyond_lin_pos(float d2, float thr, float m2r, float mr2) {
    return d2 > __fmaf_rn(thr, __fmaf_rn(thr, 1.00006103515625f, m2r), mr2);
}
// far_beyond for a threshold that cannot be negative (fmaxf(x, s) with a constant s > 0, which
// is s for a NaN x).
MD bool far_beyond_pos(float d2, float thr, float r) {
    float q = thr + r;
    return d2 > q * q * 1.00006103515625f;
}

// Weak-bound cull of a union member whose exact sphere test does not apply (an unbounded
// object, or one whose field can undercut its sphere): with l its local point, the field is at
// least c * (n - R) * scale - post, n the norm of l over the axes that do not repeat (the
// generator derives R, c and post per object). True only when that bound clears bd >= 0 by a
// relative margin of 2^-10, far beyond the rounding of either side; such a member cannot win.
MD bool weak_beyond(V l, bool ax, bool ay, bool az, float R, float c, float scl, float post, float bd) {
    float n2 = (ax ? l.x * l.x : 0.0f) + (ay ? l.y * l.y : 0.0f) + (az ? l.z * l.z : 0.0f);
    float n = sqrtf(n2);
    float lb = (n - R) * c * scl - post;
    return bd >= 0.0f && lb - (n + R) * scl * 0.0009765625f > bd;
}
// weak_beyond without the square root. In exact arithmetic its test is n > (bd + A) / K with
// K = scl (c - 2^-10) > 0 and A = post + R scl (c + 2^-10) > 0; the generator passes A rounded up
// and B = (1 + 2^-17) / K rounded up, so t = (bd + A) B exceeds the exact threshold by more than
// the few binary32 roundings of t * t, n2 and the local point (rotated with fused multiply-adds,
// rot_t_fma) can take back, and n2 > t * t implies it.
MD bool weak_beyond_sq(V l, bool ax, bool ay, bool az, float A, float B, float bd) {
    float n2 = az ? l.z * l.z : 0.0f;
    n2 = ay ? __fmaf_rn(l.y, l.y, n2) : n2;
    n2 = ax ? __fmaf_rn(l.x, l.x, n2) : n2;
    float t = (bd + A) * B;
    return bd >= 0.0f && n2 > t * t;
}

// ---- tape view ----
struct Tape {
    const TapeHeader* h;
    const DevObject* obj;
    const DevMaterial* mat;
    const DevLight* light;
    const DevSegment* seg;
    const DevNode* node;
    const uint32_t* unb;
    const DevCsgOp* csg;
    const DevVolume* vol;
};
MD Tape tape_view(const unsigned char* base) {
    Tape t;
    t.h = reinterpret_cast<const TapeHeader*>(base);
    t.obj = reinterpret_cast<const DevObject*>(base + t.h->off_objects);
    t.mat = reinterpret_cast<const DevMaterial*>(base + t.h->off_materials);
    t.light = reinterpret_cast<const DevLight*>(base + t.h->off_lights);
    t.seg = reinterpret_cast<const DevSegment*>(base + t.h->off_segments);
    t.node = reinterpret_cast<const DevNode*>(base + t.h->off_nodes);
    t.unb = reinterpret_cast<const uint32_t*>(base + t.h->off_unbounded);
    t.csg = reinterpret_cast<const DevCsgOp*>(base + t.h->off_csg);
    t.vol = reinterpret_cast<const DevVolume*>(base + t.h->off_volumes);
    return t;
}

// SdfVolume::sample (volume.rs:194-228)
MD float volume_sample(const DevVolume& v, V p) {
    if (!v.valid) return __int_as_float(0x7f800000);
    V lo = ld3(v.min), hi = ld3(v.hi), cell = ld3(v.cell);
    V c = vmin(vmax(p, lo), hi);
    float outside = length(p - c);
    V g{(c.x - lo.x) / cell.x, (c.y - lo.y) / cell.y, (c.z - lo.z) / cell.z};
    auto clampi = [](float x, uint32_t n) -> uint32_t {
        float f = fmaxf(floorf(x), 0.0f);
        uint32_t i = f >= 4294967040.0f ? 0xFFFFFFFFu : (uint32_t)f;
        return i < n - 2 ? i : n - 2;
    };
    uint32_t i0 = clampi(g.x, v.nx), j0 = clampi(g.y, v.ny), k0 = clampi(g.z, v.nz);
    float fx = clampf(g.x - (float)i0, 0.0f, 1.0f);
    float fy = clampf(g.y - (float)j0, 0.0f, 1.0f);
    float fz = clampf(g.z - (float)k0, 0.0f, 1.0f);
    const float* dd = v.data;
    size_t nx = v.nx, nxy = (size_t)v.nx * v.ny;
    size_t b = (size_t)k0 * nxy + (size_t)j0 * nx + i0;
    float c000 = __ldg(dd + b), c100 = __ldg(dd + b + 1);
    float c010 = __ldg(dd + b + nx), c110 = __ldg(dd + b + nx + 1);
    float c001 = __ldg(dd + b + nxy), c101 = __ldg(dd + b + nxy + 1);
    float c011 = __ldg(dd + b + nxy + nx), c111 = __ldg(dd + b + nxy + nx + 1);
    float x00 = c000 + (c100 - c000) * fx;
    float x10 = c010 + (c110 - c010) * fx;
    float x01 = c001 + (c101 - c001) * fx;
    float x11 = c011 + (c111 - c011) * fx;
    float y0 = x00 + (x10 - x00) * fy;
    float y1 = x01 + (x11 - x01) * fy;
    float d = y0 + (y1 - y0) * fz;
    if (!isfinite(d)) return __int_as_float(0x7f800000);
    if (outside > 0.0f) return fmaxf(outside, d - outside);
    return d;
}

// csg.rs:95-118 as a post-order stack program.
static __device__ __noinline__ float csg_eval(const DevCsgOp* op, V p) {
    float vals[MAX_CSG_STACK];
    V pts[MAX_CSG_STACK];
    int vs = 0, ps = 0;
    V cur = p;
    for (int guard = 0; guard < 4096; ++guard, ++op) {
        uint32_t o = op->op;
        if (o == CSG_OP_PRIM) {
            vals[vs++] = prim_distance(op->kind, op->p, cur);
        } else if (o == CSG_OP_XFORM) {
            pts[ps++] = cur;
            cur = scale(rot_t(op->rot, cur - ld3(op->pos)), op->inv);
        } else if (o == CSG_OP_UNXFORM) {
            cur = pts[--ps];
            vals[vs - 1] = vals[vs - 1] * op->scale;
        } else if (o == CSG_OP_UNION) {
            float b = vals[--vs];
            vals[vs - 1] = fminf(vals[vs - 1], b);
        } else if (o == CSG_OP_INTERSECT) {
            float b = vals[--vs];
            vals[vs - 1] = fmaxf(vals[vs - 1], b);
        } else if (o == CSG_OP_SUBTRACT) {
            float b = vals[--vs];
            vals[vs - 1] = fmaxf(vals[vs - 1], -b);
        } else if (o == CSG_OP_SMOOTH) {
            float b = vals[--vs];
            vals[vs - 1] = f_smooth_union(Field{vals[vs - 1], 0u}, Field{b, 0u}, op->p[0]).d;
        } else if (o == CSG_OP_OFFSET) {
            vals[vs - 1] = vals[vs - 1] - op->p[0];
        } else if (o == CSG_OP_SHELL) {
            vals[vs - 1] = fabsf(vals[vs - 1]) - op->p[0];
        } else {
            break;
        }
    }
    return vs > 0 ? vals[0] : __int_as_float(0x7f800000);
}

// sin and cos of a twist or bend angle. A scene-specialised program of a large field defines
// MM3E_SHARED_SINCOS: its objects then share one out-of-line copy of sincosf (a leaf call with
// no stack use) instead of one inlined copy per twisted or bent object, which keeps the field's
// code within the instruction cache. The values are sincosf's either way.
#if defined(MM3E_SHARED_SINCOS)
struct SinCos {
    float s, c;
};
static __device__ __noinline__ SinCos sincos_shared(float a) {
    SinCos r;
    sincosf(a, &r.s, &r.c);
    return r;
}
MD void angle_sincos(float a, float& s, float& c) {
    const SinCos r = sincos_shared(a);
    s = r.s;
    c = r.c;
}
#else
MD void angle_sincos(float a, float& s, float& c) { sincosf(a, &s, &c); }
#endif

// Object::local_point (lib.rs:400-419)
MD V local_point(const DevObject& o, V p) {
    const V d = p - ld3(o.pos);
    V r;
    if (o.flags & OF_ROT_IDENTITY) r = rot_t_identity(d);  // folded away in a specialised field
    else r = rot_t(o.rot, d);
    V l = scale(r, o.inv);
    uint32_t f = o.flags;
    if (f & OF_POINT_OPS) {
        if (f & OF_ANY_MIRROR) {
            if (f & OF_MIRROR_X) l.x = fabsf(l.x);
            if (f & OF_MIRROR_Y) l.y = fabsf(l.y);
            if (f & OF_MIRROR_Z) l.z = fabsf(l.z);
        }
        if (f & OF_ELONGATE) {
            V h = ld3(o.elongate);
            l = l - vmin(vmax(l, scale(h, -1.0f)), h);
        }
        if (f & OF_REPEAT) l = V{rep_axis(l.x, o.repeat[0]), rep_axis(l.y, o.repeat[1]), rep_axis(l.z, o.repeat[2])};
        if (f & OF_TWIST) {
            float a = o.twist * l.y;
            float s, c;
            angle_sincos(a, s, c);
            l = V{c * l.x - s * l.z, l.y, s * l.x + c * l.z};
        }
        if (f & OF_BEND) {
            float a = o.bend * l.x;
            float s, c;
            angle_sincos(a, s, c);
            l = V{c * l.x - s * l.y, s * l.x + c * l.y, l.z};
        }
    }
    return l;
}

// The tail of Object::field (lib.rs:380-397): the shape's distance d at the local point, scaled,
// rounded and onioned.
MD Field object_finish(const DevObject& o, float d) {
    d = d * o.scale;
    if (o.flags & OF_ROUND) d = d - o.round;
    if (o.flags & OF_ONION) d = fabsf(d) - o.onion;
    return Field{d, o.mat};
}

// Object::field (lib.rs:380-397)
MD Field object_field(const Tape& T, const DevObject& o, V p) {
    V l = local_point(o, p);
    float d;
    if (o.prim <= 10u) d = prim_distance(o.prim, o.params, l);
    else if (o.prim == 11u) d = csg_eval(T.csg + o.aux, l);
    else if (o.prim == 12u) d = volume_sample(T.vol[o.aux], l);
    else d = __int_as_float(0x7f800000);
    return object_finish(o, d);
}

// Register-resident traversal stack: twelve 16-bit node indices in three 64-bit words.
struct NodeStack {
    uint64_t w0, w1, w2;
    uint32_t n;
    MD void clear() { w0 = w1 = w2 = 0ull; n = 0; }
    MD void push(uint32_t x) {
        w2 = (w2 << 16) | (w1 >> 48);
        w1 = (w1 << 16) | (w0 >> 48);
        w0 = (w0 << 16) | (uint64_t)(x & 0xFFFFu);
        n += 1;
    }
    MD uint32_t pop() {
        uint32_t x = (uint32_t)(w0 & 0xFFFFull);
        w0 = (w0 >> 16) | (w1 << 48);
        w1 = (w1 >> 16) | (w2 << 48);
        w2 = w2 >> 16;
        n -= 1;
        return x;
    }
};

// Whether an exactly evaluated OF_NONCONS member's field d may lie below its bounding sphere's
// lower bound (lower, radius r) at this point, so that the BVH walk might prune the member while
// the linear fold picks it. A winner clear of its bound by a relative margin of 2^-10 cannot be
// pruned by the walk: every node on its path has a lower bound no larger than the member's
// (their spheres enclose its sphere), so a pruning best would already be below the winner.
MD bool noncons_undercut(float d, float lower, float r) { return !(d > lower + (r + fabsf(lower)) * 0.0009765625f); }

// Whether a bounded ONE segment leaves a finite accumulator `acc` exactly as it is, from its
// object's squared sphere distance d2 alone: past the slack the object's value is its sphere
// distance `lower`, and a union keeps acc when acc <= lower, a subtraction when -lower < acc,
// and a smooth union (k > 0) when lower > acc + k rounded up: then lower - acc rounds to at least
// k, the blend weight is exactly 1 and the blend returns acc bit for bit (unless acc is a zero).
// far_beyond proves lower > max(threshold, slack) in binary32 without the square root.
MD bool one_keeps_acc(uint32_t comb, float k, float acc, float d2, float r, float slack) {
    if (!(acc < __int_as_float(0x7f800000) && acc > -__int_as_float(0x7f800000))) return false;
    float thr;
    if (comb == 1u && k > 0.0f) {
        if (acc == 0.0f) return false;
        thr = __fadd_ru(acc, k);
    } else if (comb == 2u) {
        thr = -acc;
    } else {
        thr = acc;
    }
    return far_beyond(d2, fmaxf(thr, slack), r);
}

// WorldPlan::eval (accel.rs:209-252) with Bvh::query (accel.rs:79-119) and
// WorldPlan::contrib (accel.rs:187-207). The plan is walked as a generator so that the exact
// object field has a single call site: each outer iteration advances the plan to the next
// object whose exact field is needed (or none), evaluates it, and folds it with the
// reference's (distance, lowest object index) rule. ONE segments and LINEAR runs consume
// exactly one outer iteration per object on every lane, so lanes stay in step and the object
// (hence the primitive code) is warp-uniform. BVH runs walk per lane, near child first, with
// the reference's `lower > best` pruning and `lower > slack` bounding-sphere substitute; a
// LINEAR run whose winner is an exactly evaluated OF_NONCONS member that may undercut its
// bounding sphere here (noncons_undercut) falls back to that walk.
__device__ __forceinline__ Field world_eval(const Tape& T, V p) {
    const float INF = __int_as_float(0x7f800000);
    const float slack = T.h->slack;
    const uint32_t nseg = T.h->n_segments;
    enum : uint32_t { W_START = 0, W_ONE = 1, W_UNB = 2, W_BVH = 3, W_LIN = 4 };
    Field acc{INF, 0u};
    bool seeded = false;
    float bd = INF;
    int32_t bi = 0x7FFFFFFF;
    uint32_t bm = 0u;
    bool bex = false;  // the linear winner is an OF_NONCONS field that may undercut its sphere
    bool wnc = false;  // the member being evaluated is a bounded OF_NONCONS one (lower wl, radius wr)
    float wl = 0.0f, wr = 0.0f;
    uint32_t s = 0, st = W_START, ucur = 0, uend = 0, one = 0;
    NodeStack stk;
    stk.clear();
    for (int guard = 0; guard < 1 << 20; ++guard) {
        int32_t want = -1;  // object whose exact field is needed next (-1: none this step)
        bool step = false;  // this iteration consumed a uniform step (ONE / LINEAR member)
        while (want < 0 && !step) {
            if (st == W_START) {
                if (s >= nseg) return acc;
                DevSegment sg = T.seg[s];
                if (sg.kind == SEG_ONE) {
                    const DevObject& o = T.obj[sg.a];
                    one = sg.a;
                    if (o.flags & OF_BOUND) {
                        const float d2 = length_sq(p - ld3(o.bc));
                        if (seeded && one_keeps_acc(sg.b, o.k, acc.d, d2, o.br, slack)) {
                            s += 1;
                            step = true;
                            break;
                        }
                        float lower = sqrtf(d2) - o.br;
                        if (lower > slack) {
                            Field f{lower, o.mat};
                            if (!seeded) acc = f;
                            else if (sg.b == 0u) acc = f_union(acc, f);
                            else if (sg.b == 1u) acc = f_smooth_union(acc, f, o.k);
                            else acc = f_subtract(acc, f);
                            seeded = true;
                            s += 1;
                            step = true;
                            break;
                        }
                    }
                    st = W_ONE;
                    want = (int32_t)sg.a;
                    break;
                }
                bd = seeded ? acc.d : INF;
                bi = seeded ? -1 : 0x7FFFFFFF;
                bm = seeded ? acc.m : 0u;
                bex = false;
                if (sg.kind == SEG_LINEAR) {
                    ucur = sg.a;
                    uend = sg.a + sg.b;
                    st = W_LIN;
                } else {
                    ucur = sg.ua;
                    uend = sg.ua + sg.ub;
                    stk.clear();
                    if (sg.c != NIL) stk.push(sg.c);
                    st = W_UNB;
                }
            }
            if (st == W_LIN) {
                if (ucur >= uend) {
                    if (bex) {
                        // the winner may be one the BVH walk prunes: redo this run as the walk
                        DevSegment sg = T.seg[s];
                        bd = seeded ? acc.d : INF;
                        bi = seeded ? -1 : 0x7FFFFFFF;
                        bm = seeded ? acc.m : 0u;
                        ucur = sg.ua;
                        uend = sg.ua + sg.ub;
                        stk.clear();
                        if (sg.c != NIL) stk.push(sg.c);
                        st = W_UNB;
                        continue;
                    }
                    acc = Field{bd, bm};
                    seeded = true;
                    s += 1;
                    st = W_START;
                    continue;
                }
                int32_t i = (int32_t)T.unb[ucur];
                ucur += 1;
                step = true;
                const DevObject& o = T.obj[i];
                wnc = (o.flags & OF_NONCONS) && (o.flags & OF_BOUND);
                if (o.flags & OF_BOUND) {
                    const float d2 = length_sq(p - ld3(o.bc));
                    // cannot win: the squared pre-test first, without the square root (a
                    // non-conservative member past the slack as well, where its value is `lower`)
                    if (far_beyond(d2, (o.flags & OF_NONCONS) ? fmaxf(bd, slack) : bd, o.br)) break;
                    float lower = sqrtf(d2) - o.br;
                    wl = lower;
                    wr = o.br;
                    if (lower > bd && !(o.flags & OF_NONCONS)) break;  // cannot win
                    if (lower > slack) {
                        if (lower < bd || (lower == bd && i < bi)) {
                            bd = lower;
                            bi = i;
                            bm = o.mat;
                            bex = false;
                        }
                        break;
                    }
                }
                want = i;
                break;
            }
            if (st == W_UNB) {
                if (ucur < uend) {
                    want = (int32_t)T.unb[ucur];
                    ucur += 1;
                    break;
                }
                st = W_BVH;
            }
            // W_BVH
            if (stk.n == 0) {
                acc = Field{bd, bm};
                seeded = true;
                s += 1;
                st = W_START;
                continue;
            }
            const DevNode& nd = T.node[stk.pop()];
            const float nd2 = length_sq(p - V{nd.cx, nd.cy, nd.cz});
            if (far_beyond(nd2, bd, nd.r)) continue;  // lower > bd, without the square root
            float lower = sqrtf(nd2) - nd.r;
            if (lower > bd) continue;
            if (nd.leaf >= 0) {
                if (lower > slack) {
                    int32_t i = nd.leaf;
                    if (lower < bd || (lower == bd && i < bi)) {
                        bd = lower;
                        bi = i;
                        bm = T.obj[i].mat;
                    }
                    continue;
                }
                want = nd.leaf;
                break;
            }
            const DevNode& L = T.node[nd.left];
            const DevNode& R = T.node[nd.right];
            float ld = length_sq(p - V{L.cx, L.cy, L.cz});
            float rd = length_sq(p - V{R.cx, R.cy, R.cz});
            bool lnear = ld <= rd;
            stk.push(lnear ? (uint32_t)nd.right : (uint32_t)nd.left);
            stk.push(lnear ? (uint32_t)nd.left : (uint32_t)nd.right);
        }
        if (want < 0) continue;
        Field f = object_field(T, T.obj[want], p);
        if (st == W_ONE) {
            uint32_t comb = (T.obj[one].flags >> 16) & 3u;
            if (!seeded) acc = f;
            else if (comb == 0u) acc = f_union(acc, f);
            else if (comb == 1u) acc = f_smooth_union(acc, f, T.obj[one].k);
            else acc = f_subtract(acc, f);
            seeded = true;
            s += 1;
            st = W_START;
        } else if (f.d < bd || (f.d == bd && want < bi)) {
            bd = f.d;
            bi = want;
            bm = f.m;
            bex = st == W_LIN && wnc && noncons_undercut(f.d, wl, wr);
        }
    }
    return acc;
}

// One plain-union run of the plan walked as Bvh::query (accel.rs:79-119): its unbounded
// members first, then the sphere BVH near child first with the `lower > best` prune and the
// `lower > slack` bounding-sphere substitute, folded into `acc` by (distance, lowest index).
// The same steps as world_eval's W_UNB / W_BVH states, as one call for the scene-specialised
// field (big runs, and LINEAR runs whose winner may undercut its bound).
static __device__ __noinline__ Field bvh_segment(const Tape& T, uint32_t s, V p, bool seeded, Field acc) {
    const float INF = __int_as_float(0x7f800000);
    const float slack = T.h->slack;
    DevSegment sg = T.seg[s];
    float bd = seeded ? acc.d : INF;
    int32_t bi = seeded ? -1 : 0x7FFFFFFF;
    uint32_t bm = seeded ? acc.m : 0u;
    for (uint32_t u = sg.ua; u < sg.ua + sg.ub; ++u) {
        int32_t i = (int32_t)T.unb[u];
        Field f = object_field(T, T.obj[i], p);
        if (f.d < bd || (f.d == bd && i < bi)) {
            bd = f.d;
            bi = i;
            bm = f.m;
        }
    }
    NodeStack stk;
    stk.clear();
    if (sg.c != NIL) stk.push(sg.c);
    while (stk.n > 0) {
        const DevNode& nd = T.node[stk.pop()];
        const float nd2 = length_sq(p - V{nd.cx, nd.cy, nd.cz});
        if (far_beyond(nd2, bd, nd.r)) continue;  // lower > bd, without the square root
        float lower = sqrtf(nd2) - nd.r;
        if (lower > bd) continue;
        if (nd.leaf >= 0) {
            int32_t i = nd.leaf;
            if (lower > slack) {
                if (lower < bd || (lower == bd && i < bi)) {
                    bd = lower;
                    bi = i;
                    bm = T.obj[i].mat;
                }
                continue;
            }
            Field f = object_field(T, T.obj[i], p);
            if (f.d < bd || (f.d == bd && i < bi)) {
                bd = f.d;
                bi = i;
                bm = f.m;
            }
            continue;
        }
        const DevNode& L = T.node[nd.left];
        const DevNode& R = T.node[nd.right];
        float ld = length_sq(p - V{L.cx, L.cy, L.cz});
        float rd = length_sq(p - V{R.cx, R.cy, R.cz});
        bool lnear = ld <= rd;
        stk.push(lnear ? (uint32_t)nd.right : (uint32_t)nd.left);
        stk.push(lnear ? (uint32_t)nd.left : (uint32_t)nd.right);
    }
    return Field{bd, bm};
}

// ---- dual numbers (dual.rs) for the exact-gradient normal of dual-safe scenes ----
struct D {
    float v;
    V g;
};
MD D dc(float v) { return D{v, V{0.f, 0.f, 0.f}}; }
MD D dscale(D a, float s) { return D{a.v * s, scale(a.g, s)}; }
MD D dadds(D a, float s) { return D{a.v + s, a.g}; }
MD D dneg(D a) { return D{-a.v, -a.g}; }
MD D dabs(D a) { return a.v >= 0.0f ? a : dneg(a); }
MD D dsqrt(D a) {
    float v = sqrtf(fmaxf(a.v, 0.0f));
    float k = v > 1e-9f ? 0.5f / v : 0.0f;
    return D{v, scale(a.g, k)};
}
MD D dmin(D a, D o) { return a.v <= o.v ? a : o; }
MD D dmax(D a, D o) { return a.v >= o.v ? a : o; }
MD D dmax0(D a) { return dmax(a, dc(0.0f)); }
MD D dmaxc(D a, float c) { return a.v >= c ? a : dc(c); }
MD D dclamp(D a, float lo, float hi) { return dmin(dmax(a, dc(lo)), dc(hi)); }
MD D dadd(D a, D o) { return D{a.v + o.v, a.g + o.g}; }
MD D dsub(D a, D o) { return D{a.v - o.v, a.g - o.g}; }
MD D dmul(D a, D o) { return D{a.v * o.v, scale(a.g, o.v) + scale(o.g, a.v)}; }
MD D ddiv(D a, D o) {
    float inv2 = 1.0f / (o.v * o.v);
    return D{a.v / o.v, scale(scale(a.g, o.v) - scale(o.g, a.v), inv2)};
}
MD D dd_box(D x, D y, D z, V half) {
    D qx = dadds(dabs(x), -half.x), qy = dadds(dabs(y), -half.y), qz = dadds(dabs(z), -half.z);
    D out = dsqrt(dadd(dadd(dmul(dmax0(qx), dmax0(qx)), dmul(dmax0(qy), dmax0(qy))), dmul(dmax0(qz), dmax0(qz))));
    D in = dmin(dmax(qx, dmax(qy, qz)), dc(0.0f));
    return dadd(out, in);
}
// Prim::distance_dual (lib.rs:244-261; dual.rs:129-232). Inlined where the primitive is a
// compile-time constant (a scene-specialised program); called through prim_dual elsewhere.
MD D prim_dual_inl(uint32_t kind, const float* q, D x, D y, D z) {
    switch (kind) {
        case 0: return dadds(dsqrt(dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z))), -q[0]);
        case 1: return dd_box(x, y, z, V{q[0], q[1], q[2]});
        case 2: return dadds(dd_box(x, y, z, V{q[0], q[1], q[2]} - splat(q[3])), -q[3]);
        case 3: {
            D t = dadds(dsqrt(dadd(dmul(x, x), dmul(z, z))), -q[0]);
            return dadds(dsqrt(dadd(dmul(t, t), dmul(y, y))), -q[1]);
        }
        case 4: {
            D dx = dadds(dsqrt(dadd(dmul(x, x), dmul(z, z))), -q[1]);
            D dy = dadds(dabs(y), -q[0]);
            D in = dmin(dmax(dx, dy), dc(0.0f));
            D ox = dmax0(dx), oy = dmax0(dy);
            return dadd(in, dsqrt(dadd(dmul(ox, ox), dmul(oy, oy))));
        }
        case 5: {
            V a{q[0], q[1], q[2]}, b{q[3], q[4], q[5]};
            D pax = dadds(x, -a.x), pay = dadds(y, -a.y), paz = dadds(z, -a.z);
            V ba = b - a;
            float dbb = fmaxf(dot(ba, ba), 1e-12f);
            D dpb = dadd(dadd(dscale(pax, ba.x), dscale(pay, ba.y)), dscale(paz, ba.z));
            D hh = dclamp(dscale(dpb, 1.0f / dbb), 0.0f, 1.0f);
            D rx = dsub(pax, dscale(hh, ba.x)), ry = dsub(pay, dscale(hh, ba.y)), rz = dsub(paz, dscale(hh, ba.z));
            return dadds(dsqrt(dadd(dadd(dmul(rx, rx), dmul(ry, ry)), dmul(rz, rz))), -q[6]);
        }
        case 6: {
            float r1 = q[0], r2 = q[1], h = q[2];
            D qx = dsqrt(dadd(dmul(x, x), dmul(z, z)));
            D qy = y;
            float b = (r1 - r2) / fmaxf(h, 1e-6f);
            float a = sqrtf(fmaxf(1.0f - b * b, 0.0f));
            D k = dadd(dscale(qx, -b), dscale(qy, a));
            if (k.v < 0.0f) return dadds(dsqrt(dadd(dmul(qx, qx), dmul(qy, qy))), -r1);
            if (k.v > a * h) {
                D qyh = dadds(qy, -h);
                return dadds(dsqrt(dadd(dmul(qx, qx), dmul(qyh, qyh))), -r2);
            }
            return dadds(dadd(dscale(qx, a), dscale(qy, b)), -r1);
        }
        case 7: {
            V r{q[0], q[1], q[2]};
            D k0x = dscale(x, 1.0f / r.x), k0y = dscale(y, 1.0f / r.y), k0z = dscale(z, 1.0f / r.z);
            D k0 = dsqrt(dadd(dadd(dmul(k0x, k0x), dmul(k0y, k0y)), dmul(k0z, k0z)));
            if (k0.v < 1e-6f) return dc(-fminf(fminf(r.x, r.y), r.z));
            D k1x = dscale(x, 1.0f / (r.x * r.x)), k1y = dscale(y, 1.0f / (r.y * r.y)), k1z = dscale(z, 1.0f / (r.z * r.z));
            D k1 = dmaxc(dsqrt(dadd(dadd(dmul(k1x, k1x), dmul(k1y, k1y)), dmul(k1z, k1z))), 1e-9f);
            return ddiv(dmul(k0, dadds(k0, -1.0f)), k1);
        }
        case 8: return dscale(dadds(dadd(dadd(dabs(x), dabs(y)), dabs(z)), -q[0]), 0.5773503f);
        case 9: {
            const float kx = -0.8660254f, ky = 0.5f, kz = 0.57735f;
            float r = q[0], h = q[1];
            D ax0 = dabs(x), az0 = dabs(z);
            D ay = dadds(dabs(y), -h);
            D t = dscale(dmin(dadd(dscale(ax0, kx), dscale(az0, ky)), dc(0.0f)), 2.0f);
            D ax = dsub(ax0, dscale(t, kx)), az = dsub(az0, dscale(t, ky));
            D cl = dclamp(ax, -kz * r, kz * r);
            D dfx = dsub(ax, cl), dfz = dadds(az, -r);
            float sg = dfz.v >= 0.0f ? 1.0f : -1.0f;
            D dx = dscale(dsqrt(dadd(dmul(dfx, dfx), dmul(dfz, dfz))), sg);
            D in = dmin(dmax(dx, ay), dc(0.0f));
            D ox = dmax0(dx), oy = dmax0(ay);
            return dadd(in, dsqrt(dadd(dmul(ox, ox), dmul(oy, oy))));
        }
        case 10: return dadds(dadd(dadd(dscale(x, q[0]), dscale(y, q[1])), dscale(z, q[2])), q[3]);
        default: return dc(__int_as_float(0x7f800000));
    }
}
static __device__ __noinline__ D prim_dual(uint32_t kind, const float* q, D x, D y, D z) {
    return prim_dual_inl(kind, q, x, y, z);
}
// Object::field_dual (lib.rs:435-463); INL inlines the primitive (a constant object record).
template <bool INL = false>
MD D object_dual(const DevObject& o, V p) {
    D wx{p.x, V{1.f, 0.f, 0.f}}, wy{p.y, V{0.f, 1.f, 0.f}}, wz{p.z, V{0.f, 0.f, 1.f}};
    D tx = dadds(wx, -o.pos[0]), ty = dadds(wy, -o.pos[1]), tz = dadds(wz, -o.pos[2]);
    const float* r = o.rot;
    D lx = dscale(dadd(dadd(dscale(tx, r[0]), dscale(ty, r[1])), dscale(tz, r[2])), o.inv);
    D ly = dscale(dadd(dadd(dscale(tx, r[3]), dscale(ty, r[4])), dscale(tz, r[5])), o.inv);
    D lz = dscale(dadd(dadd(dscale(tx, r[6]), dscale(ty, r[7])), dscale(tz, r[8])), o.inv);
    uint32_t f = o.flags;
    if (f & OF_MIRROR_X) lx = dabs(lx);
    if (f & OF_MIRROR_Y) ly = dabs(ly);
    if (f & OF_MIRROR_Z) lz = dabs(lz);
    if (f & OF_ELONGATE) {
        D cx = dclamp(lx, -o.elongate[0], o.elongate[0]);
        D cy = dclamp(ly, -o.elongate[1], o.elongate[1]);
        D cz = dclamp(lz, -o.elongate[2], o.elongate[2]);
        lx = dsub(lx, cx);
        ly = dsub(ly, cy);
        lz = dsub(lz, cz);
    }
    if (f & OF_REPEAT) {
        if (o.repeat[0] > 0.0f) lx = dadds(lx, -roundf(lx.v / o.repeat[0]) * o.repeat[0]);
        if (o.repeat[1] > 0.0f) ly = dadds(ly, -roundf(ly.v / o.repeat[1]) * o.repeat[1]);
        if (o.repeat[2] > 0.0f) lz = dadds(lz, -roundf(lz.v / o.repeat[2]) * o.repeat[2]);
    }
    D d = dscale(INL ? prim_dual_inl(o.prim, o.params, lx, ly, lz) : prim_dual(o.prim, o.params, lx, ly, lz), o.scale);
    if (f & OF_ROUND) d = dadds(d, -o.round);
    if (f & OF_ONION) d = dadds(dabs(d), -o.onion);
    return d;
}
// One fold step of Scene::normal_dual (lib.rs:820-835): combine mode in flags bits 16-17.
MD D dual_fold(D acc, D f, uint32_t flags, float k) {
    uint32_t comb = (flags >> 16) & 3u;
    if (comb == 0u) return dmin(acc, f);
    if (comb == 1u) {
        if (k <= 0.0f) return dmin(acc, f);
        D h = dclamp(dadds(dscale(dsub(f, acc), 0.5f / k), 0.5f), 0.0f, 1.0f);
        D omh = dsub(dc(1.0f), h);
        return dsub(dadd(dmul(f, omh), dmul(acc, h)), dscale(dmul(h, omh), k));
    }
    return dmax(acc, dneg(f));
}
// Scene::normal_dual (lib.rs:820-835): every object, no pruning.
static __device__ __noinline__ V normal_dual(const DevObject* objs, uint32_t n, V p) {
    if (n == 0) return V{0.f, 0.f, 0.f};
    D acc = object_dual(objs[0], p);
    for (uint32_t i = 1; i < n; ++i) {
        const DevObject& o = objs[i];
        acc = dual_fold(acc, object_dual(o, p), o.flags, o.k);
    }
    return normalize(acc.g);
}

// ---- shade.rs ----
MD float fresnel_schlick(float c, float f0) { return f0 + (1.0f - f0) * powi5(clampf(1.0f - c, 0.0f, 1.0f)); }
MD float luminance(V c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }
MD V brdf(V n, V l, V view, V albedo, float metallic, float roughness, float reflectance) {  // shade.rs:51-72
    float nol = fmaxf(dot(n, l), 0.0f);
    if (nol <= 0.0f) return V{0.f, 0.f, 0.f};
    float nov = fmaxf(dot(n, view), 1e-4f);
    V h = normalize(l + view);
    float noh = fmaxf(dot(n, h), 0.0f);
    float voh = fmaxf(dot(view, h), 0.0f);
    float a = fmaxf(roughness * roughness, 1e-3f);
    float a2 = a * a;
    V f0 = mix(splat(0.08f * clampf(reflectance, 0.0f, 1.0f)), albedo, metallic);
    float m5 = powi5(clampf(1.0f - voh, 0.0f, 1.0f));
    V f = f0 + scale(splat(1.0f) - f0, m5);
    const float PI = 3.14159265358979323846f;
    float dn = noh * noh * (a2 - 1.0f) + 1.0f;
    float dg = a2 / fmaxf(PI * dn * dn, 1e-12f);
    float gv = nol * sqrtf(nov * nov * (1.0f - a2) + a2);
    float gl = nov * sqrtf(nol * nol * (1.0f - a2) + a2);
    float vs = 0.5f / fmaxf(gv + gl, 1e-5f);
    V spec = scale(f, dg * vs);
    V kd = scale(splat(1.0f) - f, 1.0f - metallic);
    V diff = scale(cmul(kd, albedo), 1.0f / PI);
    return scale(diff + spec, nol);
}
MD V sky_base(V dir) {
    float t = clampf(0.5f * (dir.y + 1.0f), 0.0f, 1.0f);
    return mix(V{0.78f, 0.86f, 0.96f}, V{0.20f, 0.38f, 0.72f}, t);
}
MD V sky(V dir, V sun) {  // shade.rs:76-84
    V base = sky_base(dir);
    float s = fmaxf(dot(dir, sun), 0.0f);
    float glow = powf(s, 8.0f) * 0.3f + powf(s, 220.0f) * 6.0f;
    return base + splat(glow);
}
MD V sky_diffuse(V dir, V sun) {  // shade.rs:88-95
    V base = sky_base(dir);
    float soft = powf(fmaxf(dot(dir, sun), 0.0f), 8.0f) * 0.3f;
    return base + splat(soft);
}
MD float aces1(float v) {
    v = fmaxf(v, 0.0f);
    return clampf((v * (2.51f * v + 0.03f)) / (v * (2.43f * v + 0.59f) + 0.14f), 0.0f, 1.0f);
}
MD V display(V c, float exposure) {  // post.rs:306-307: clamp01(gamma(aces(c * exposure)))
    V x = scale(c, exposure);
    const float inv = 1.0f / 2.2f;
    V a{aces1(x.x), aces1(x.y), aces1(x.z)};
    return clamp01(V{powf(fmaxf(a.x, 0.0f), inv), powf(fmaxf(a.y, 0.0f), inv), powf(fmaxf(a.z, 0.0f), inv)});
}
MD V apply_fog(V c, V fog, float t, float density) {  // shade.rs:113-116
    float f = 1.0f - expf(-t * density);
    return mix(c, fog, clampf(f, 0.0f, 1.0f));
}

// FNV-1a hash_cell (mm3e-kit/src/lib.rs:63-78)
MD float hash_cell(int32_t ix, int32_t iy) {
    uint64_t h = 0xcbf29ce484222325ull;
    uint32_t ux = (uint32_t)ix, uy = (uint32_t)iy;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        h ^= (uint64_t)((ux >> (8 * i)) & 0xFFu);
        h *= 0x00000100000001b3ull;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        h ^= (uint64_t)((uy >> (8 * i)) & 0xFFu);
        h *= 0x00000100000001b3ull;
    }
    return (float)(h >> 40) / 16777216.0f;
}
MD int32_t f2i_sat(float x) {  // Rust `as i32`
    return __float2int_rz(x);  // saturates, NaN -> 0
}
// surface_albedo (lib.rs:1365-1375)
MD V surface_albedo(const DevMaterial& m, V p) {
    V alb = ld3(m.albedo);
    if (!m.checker) return alb;
    int32_t ix = f2i_sat(floorf(p.x)), iz = f2i_sat(floorf(p.z));
    int32_t sum = (int32_t)((uint32_t)ix + (uint32_t)iz);
    int32_t rem = sum % 2;
    if (rem < 0) rem += 2;
    V base = rem == 0 ? splat(0.92f) : splat(0.20f);
    float tint = hash_cell(ix, iz) * 0.06f - 0.03f;
    return max_scalar(cmul(base + splat(tint), alb), 0.0f);
}
// ibl_irradiance (lib.rs:1379-1398)
MD V ibl_irradiance(V n, V sun, V sky_ambient) {
    V up = fabsf(n.y) > 0.9f ? V{1.f, 0.f, 0.f} : V{0.f, 1.f, 0.f};
    V t1 = normalize(cross(n, up));
    V t2 = normalize(cross(n, t1));
    V n6 = scale(n, 0.6f);
    V acc{0.f, 0.f, 0.f};
    float w = 0.0f;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        V d = i == 0 ? n
              : i == 1 ? normalize(n6 + scale(t1, 0.6f))
              : i == 2 ? normalize(n6 - scale(t1, 0.6f))
              : i == 3 ? normalize(n6 + scale(t2, 0.6f))
                       : normalize(n6 - scale(t2, 0.6f));
        float cw = fmaxf(dot(d, n), 0.0f);
        acc = acc + scale(sky_diffuse(d, sun), cw);
        w = w + cw;
    }
    return cmul(scale(acc, 1.0f / fmaxf(w, 1e-4f)), sky_ambient);
}
// GiVolume::sample (gi.rs:138-187); cubes are float4 per face.
MD V gi_sample(const TapeHeader& h, V pos, V n) {
    auto axis = [](float p, float lo, float ext, uint32_t nn) {
        return fabsf(ext) > 1e-6f ? (p - lo) / ext * (float)((nn > 2u ? nn : 2u) - 1u) : 0.0f;
    };
    V g{axis(pos.x, h.gi_min[0], h.gi_size[0], h.gi_nx), axis(pos.y, h.gi_min[1], h.gi_size[1], h.gi_ny),
        axis(pos.z, h.gi_min[2], h.gi_size[2], h.gi_nz)};
    auto clampi = [](float v, uint32_t hi) -> uint32_t {
        float f = fmaxf(floorf(v), 0.0f);
        uint32_t i = f >= 4294967040.0f ? 0xFFFFFFFFu : (uint32_t)f;
        uint32_t top = hi > 0u ? hi - 1u : 0u;
        return i < top ? i : top;
    };
    uint32_t nx = h.gi_nx, ny = h.gi_ny, nz = h.gi_nz;
    uint32_t i0 = clampi(g.x, nx), j0 = clampi(g.y, ny), k0 = clampi(g.z, nz);
    uint32_t i1 = min(i0 + 1u, nx - 1u), j1 = min(j0 + 1u, ny - 1u), k1 = min(k0 + 1u, nz - 1u);
    float fx = clampf(g.x - (float)i0, 0.0f, 1.0f);
    float fy = clampf(g.y - (float)j0, 0.0f, 1.0f);
    float fz = clampf(g.z - (float)k0, 0.0f, 1.0f);
    // Only the three faces the normal selects are needed (per-face interpolation is independent).
    int faces[3] = {n.x >= 0.0f ? 0 : 1, n.y >= 0.0f ? 2 : 3, n.z >= 0.0f ? 4 : 5};
    V res[3];
    const float4* cubes = h.gi_cubes;
    auto at = [&](uint32_t i, uint32_t j, uint32_t k, int f) {
        float4 c = __ldg(cubes + ((size_t)((size_t)k * ny + j) * nx + i) * 6 + f);
        return V{c.x, c.y, c.z};
    };
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        int f = faces[q];
        V x00 = mix(at(i0, j0, k0, f), at(i1, j0, k0, f), fx);
        V x10 = mix(at(i0, j1, k0, f), at(i1, j1, k0, f), fx);
        V x01 = mix(at(i0, j0, k1, f), at(i1, j0, k1, f), fx);
        V x11 = mix(at(i0, j1, k1, f), at(i1, j1, k1, f), fx);
        res[q] = mix(mix(x00, x10, fy), mix(x01, x11, fy), fz);
    }
    V nn{n.x * n.x, n.y * n.y, n.z * n.z};
    return scale(res[0], nn.x) + scale(res[1], nn.y) + scale(res[2], nn.z);
}

// Light::{toward, attenuation, shadow_k} (lib.rs:529-556)
MD void light_toward(const DevLight& l, V p, V& dir, float& dist) {
    if (l.directional) {
        dir = ld3(l.vec);
        dist = __int_as_float(0x7f800000);
    } else {
        V d = ld3(l.vec) - p;
        float len = length(d);
        dir = scale(d, 1.0f / fmaxf(len, 1e-6f));
        dist = len;
    }
}
MD float light_atten(const DevLight& l, float dist) {
    if (l.directional) return 1.0f;
    float m = fmaxf(dist, 0.05f);
    return 1.0f / (m * m);
}
MD float light_shadow_k(const DevLight& l, float dist) {
    if (l.radius <= 0.0f) return 24.0f;
    if (l.directional) return clampf(1.0f / l.radius, 2.0f, 64.0f);
    return clampf(dist / l.radius, 2.0f, 64.0f);
}

}  // namespace mm3e
