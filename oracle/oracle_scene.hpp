// oracle_scene.hpp — restatement of the MM3E orchestrator render path
// (mm3e-orchestrator/src/{lib.rs, accel.rs, gi.rs, post.rs, appearance.rs}).
//
// TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline for the CUDA path.
// It consumes the same flat `mm3e_scene_desc` that the C ABI takes, so both sides see
// bit-identical inputs. Operation order follows the Rust source line by line.
#pragma once
#include <algorithm>
#include <array>
#include <optional>
#include <string>
#include <thread>
#include <vector>

#include "../include/mm3e_cuda.h"
#include "oracle_kit.hpp"

namespace oracle {

// color.rs:153-162
template <class T> struct Material {
    V3<T> albedo{T(0), T(0), T(0)};
    T metallic = T(0), specular = T(0), roughness = T(0), reflectivity = T(0);
    V3<T> emissive{T(0), T(0), T(0)};
    bool checker = false;
};

// lib.rs:503-557
template <class T> struct Light {
    V3<T> vec, color;
    bool directional = true;
    T radius = T(0);
    // lib.rs:529-537
    void toward(V3<T> p, V3<T>& dir, T& dist) const {
        if (directional) {
            dir = vec;
            dist = o_inf<T>();
        } else {
            V3<T> d = vec - p;
            T len = length(d);
            dir = scale(d, T(1) / o_max(len, OL(1e-6)));
            dist = len;
        }
    }
    // lib.rs:539-545
    T attenuation(T dist) const {
        if (directional) return T(1);
        T m = o_max(dist, OL(0.05));
        return T(1) / (m * m);
    }
    // lib.rs:547-556
    T shadow_k(T dist) const {
        if (radius <= T(0)) return T(24);
        if (directional) return o_clamp(T(1) / radius, T(2), T(64));
        return o_clamp(dist / radius, T(2), T(64));
    }
};

// lib.rs:330-336 + Modifiers (lib.rs:311-319)
template <class T> struct Object {
    uint32_t prim = 0, id = 0, mat = 0, combine = 0;
    T k = T(0);
    T p[7] = {};
    Xform<T> xf;
    bool mx = false, my = false, mz = false;
    V3<T> repeat{T(0), T(0), T(0)};
    T twist = T(0), bend = T(0);
    V3<T> elongate{T(0), T(0), T(0)};
    T round = T(0), onion = T(0);
    bool any_mirror() const { return mx || my || mz; }
};

// post.rs:14-29
template <class T> struct Post {
    T exposure = T(1);
    bool bloom = true;
    T threshold = T(1), intensity = OL(0.06);
    uint32_t radius = 12;
};

// gi.rs:17-23
template <class T> struct GiVolume {
    V3<T> min, size;
    uint64_t nx = 1, ny = 1, nz = 1;
    std::vector<std::array<V3<T>, 6>> cubes;
    const std::array<V3<T>, 6>& cube_at(uint64_t i, uint64_t j, uint64_t k) const { return cubes[(k * ny + j) * nx + i]; }
    // gi.rs:138-187
    V3<T> sample(V3<T> pos, V3<T> n) const {
        auto axis = [](T p, T lo, T ext, uint64_t nn) {
            if (o_abs(ext) > OL(1e-6)) return (p - lo) / ext * T((float)((nn > 2 ? nn : 2) - 1));
            return T(0);
        };
        V3<T> g{axis(pos.x, min.x, size.x, nx), axis(pos.y, min.y, size.y, ny), axis(pos.z, min.z, size.z, nz)};
        auto clampi = [](T v, uint64_t hi) {
            uint64_t i = o_to_usize(o_max(o_floor(v), T(0)));
            uint64_t top = hi > 0 ? hi - 1 : 0;
            return i < top ? i : top;
        };
        uint64_t i0 = clampi(g.x, nx), j0 = clampi(g.y, ny), k0 = clampi(g.z, nz);
        uint64_t i1 = std::min(i0 + 1, nx - 1), j1 = std::min(j0 + 1, ny - 1), k1 = std::min(k0 + 1, nz - 1);
        T fx = o_clamp(g.x - T((float)i0), T(0), T(1));
        T fy = o_clamp(g.y - T((float)j0), T(0), T(1));
        T fz = o_clamp(g.z - T((float)k0), T(0), T(1));
        V3<T> face[6];
        for (int f = 0; f < 6; ++f) {
            V3<T> c000 = cube_at(i0, j0, k0)[f], c100 = cube_at(i1, j0, k0)[f];
            V3<T> c010 = cube_at(i0, j1, k0)[f], c110 = cube_at(i1, j1, k0)[f];
            V3<T> c001 = cube_at(i0, j0, k1)[f], c101 = cube_at(i1, j0, k1)[f];
            V3<T> c011 = cube_at(i0, j1, k1)[f], c111 = cube_at(i1, j1, k1)[f];
            V3<T> x00 = mix(c000, c100, fx), x10 = mix(c010, c110, fx);
            V3<T> x01 = mix(c001, c101, fx), x11 = mix(c011, c111, fx);
            V3<T> y0 = mix(x00, x10, fy), y1 = mix(x01, x11, fy);
            face[f] = mix(y0, y1, fz);
        }
        V3<T> nn{n.x * n.x, n.y * n.y, n.z * n.z};
        V3<T> fxf = n.x >= T(0) ? face[0] : face[1];
        V3<T> fyf = n.y >= T(0) ? face[2] : face[3];
        V3<T> fzf = n.z >= T(0) ? face[4] : face[5];
        return scale(fxf, nn.x) + scale(fyf, nn.y) + scale(fzf, nn.z);
    }
};

// lib.rs:561-620
template <class T> struct Scene {
    uint32_t width = 0, height = 0;
    std::vector<Object<T>> objects;
    std::vector<Material<T>> materials;
    std::vector<Light<T>> lights;
    V3<T> sun_dir, ambient, sky_ambient, fog;
    T fog_density = T(0);
    uint32_t aa = 1, bounces = 0;
    bool shadows = true, ao = true;
    Marcher<T> marcher;
    Post<T> post;
    uint32_t mode = MM3E_MODE_BEAUTY;
    std::optional<GiVolume<T>> gi;
    std::vector<Volume<T>> volumes;
    std::vector<CsgNode<T>> csg_nodes;
    std::vector<uint32_t> csg_roots;
};

template <class T> inline V3<T> v3f(const float* a) { return V3<T>{T(a[0]), T(a[1]), T(a[2])}; }

// Convert the C-ABI description (f32) into the oracle's scalar type.
template <class T> inline Scene<T> scene_from_desc(const mm3e_scene_desc& d) {
    Scene<T> s;
    s.width = d.width;
    s.height = d.height;
    for (uint32_t i = 0; i < d.n_objects; ++i) {
        const mm3e_object& o = d.objects[i];
        Object<T> ob;
        ob.prim = o.prim;
        ob.id = o.id;
        ob.mat = o.mat;
        ob.combine = o.combine;
        ob.k = T(o.smooth_k);
        for (int j = 0; j < 7; ++j) ob.p[j] = T(o.params[j]);
        for (int c = 0; c < 3; ++c) ob.xf.rot.c[c] = v3f<T>(o.rot + 3 * c);
        ob.xf.pos = v3f<T>(o.pos);
        ob.xf.scale = T(o.scale);
        ob.mx = (o.mirror & 1u) != 0;
        ob.my = (o.mirror & 2u) != 0;
        ob.mz = (o.mirror & 4u) != 0;
        ob.repeat = v3f<T>(o.repeat);
        ob.twist = T(o.twist);
        ob.bend = T(o.bend);
        ob.elongate = v3f<T>(o.elongate);
        ob.round = T(o.round);
        ob.onion = T(o.onion);
        s.objects.push_back(ob);
    }
    for (uint32_t i = 0; i < d.n_materials; ++i) {
        const mm3e_material& m = d.materials[i];
        Material<T> mt;
        mt.albedo = v3f<T>(m.albedo);
        mt.metallic = T(m.metallic);
        mt.specular = T(m.specular);
        mt.roughness = T(m.roughness);
        mt.reflectivity = T(m.reflectivity);
        mt.emissive = v3f<T>(m.emissive);
        mt.checker = m.checker != 0;
        s.materials.push_back(mt);
    }
    for (uint32_t i = 0; i < d.n_lights; ++i) {
        const mm3e_light& l = d.lights[i];
        Light<T> lt;
        lt.vec = v3f<T>(l.vec);
        lt.color = v3f<T>(l.color);
        lt.directional = l.directional != 0;
        lt.radius = T(l.radius);
        s.lights.push_back(lt);
    }
    s.sun_dir = v3f<T>(d.sun_dir);
    s.ambient = v3f<T>(d.ambient);
    s.sky_ambient = v3f<T>(d.sky_ambient);
    s.fog = v3f<T>(d.fog);
    s.fog_density = T(d.fog_density);
    s.aa = d.aa;
    s.bounces = d.bounces;
    s.shadows = d.shadows != 0;
    s.ao = d.ao != 0;
    s.marcher.max_steps = d.marcher.max_steps;
    s.marcher.max_dist = T(d.marcher.max_dist);
    s.marcher.eps = T(d.marcher.eps);
    s.marcher.step_scale = T(d.marcher.step_scale);
    s.marcher.shadow_steps = d.marcher.shadow_steps;
    s.marcher.ao_samples = d.marcher.ao_samples;
    s.marcher.lod_footprint = T(d.marcher.lod_footprint);
    s.marcher.subitize = T(d.marcher.subitize);
    s.marcher.secant = d.marcher.secant != 0;
    s.marcher.normal_h = T(d.marcher.normal_h);
    s.post.exposure = T(d.post.exposure);
    s.post.bloom = d.post.bloom != 0;
    s.post.threshold = T(d.post.bloom_threshold);
    s.post.intensity = T(d.post.bloom_intensity);
    s.post.radius = d.post.bloom_radius;
    s.mode = d.mode;
    if (d.gi) {
        GiVolume<T> g;
        g.min = v3f<T>(d.gi->min);
        g.size = v3f<T>(d.gi->size);
        g.nx = d.gi->nx;
        g.ny = d.gi->ny;
        g.nz = d.gi->nz;
        uint64_t n = g.nx * g.ny * g.nz;
        g.cubes.resize(n);
        for (uint64_t i = 0; i < n; ++i)
            for (int f = 0; f < 6; ++f) g.cubes[i][f] = v3f<T>(d.gi->cubes + i * 18 + f * 3);
        s.gi = g;
    }
    for (uint32_t i = 0; i < d.n_volumes; ++i) {
        const mm3e_volume& v = d.volumes[i];
        Volume<T> vol;
        vol.nx = v.nx;
        vol.ny = v.ny;
        vol.nz = v.nz;
        vol.min = v3f<T>(v.min);
        vol.cell = v3f<T>(v.cell);
        uint64_t n = (uint64_t)v.nx * v.ny * v.nz;
        vol.data.resize(n);
        for (uint64_t j = 0; j < n; ++j) vol.data[j] = T(v.data[j]);
        s.volumes.push_back(std::move(vol));
    }
    for (uint32_t i = 0; i < d.n_csg_nodes; ++i) {
        const mm3e_csg_node& n = d.csg_nodes[i];
        CsgNode<T> c;
        c.kind = n.kind;
        c.a = n.a;
        c.b = n.b;
        for (int j = 0; j < 7; ++j) c.p[j] = T(n.params[j]);
        for (int k = 0; k < 3; ++k) c.xf.rot.c[k] = v3f<T>(n.rot + 3 * k);
        c.xf.pos = v3f<T>(n.pos);
        c.xf.scale = T(n.scale);
        s.csg_nodes.push_back(c);
    }
    for (uint32_t i = 0; i < d.n_csgs; ++i) s.csg_roots.push_back(d.csg_roots[i]);
    return s;
}

// ------------------------------------------------------------------------------------------
// Object geometry (lib.rs:214-293, 380-496)
// ------------------------------------------------------------------------------------------

// Prim::distance (lib.rs:215-241)
template <class T> inline T object_prim_distance(const Scene<T>& s, const Object<T>& o, V3<T> local) {
    if (o.prim == K_CSG) return csg_distance(s.csg_nodes, s.csg_roots[o.id], local);
    if (o.prim == K_VOLUME) {
        if (s.volumes.empty()) return o_inf<T>();
        return s.volumes[o.id % s.volumes.size()].sample(local);
    }
    return prim_distance(o.prim, o.p, local);
}

// Prim::local_bound (lib.rs:264-292)
template <class T> inline bool prim_local_bound(const Scene<T>& s, const Object<T>& o, V3<T>& c, T& r) {
    const T* q = o.p;
    switch (o.prim) {
        case K_SPHERE: c = zero3<T>(); r = q[0]; return true;
        case K_BOX: case K_ROUND_BOX: c = zero3<T>(); r = length(V3<T>{q[0], q[1], q[2]}); return true;
        case K_TORUS: c = zero3<T>(); r = q[0] + q[1]; return true;
        case K_CYLINDER: c = zero3<T>(); r = o_sqrt(q[0] * q[0] + q[1] * q[1]); return true;
        case K_CAPSULE: {
            V3<T> a{q[0], q[1], q[2]}, b{q[3], q[4], q[5]};
            c = scale(a + b, OL(0.5));
            r = length(scale(a - b, OL(0.5))) + q[6];
            return true;
        }
        case K_CONE:
            c = V3<T>{T(0), q[2] * OL(0.5), T(0)};
            r = o_max(o_max(q[2] * OL(0.5) + o_max(q[0], q[1]), q[0]), q[1]);
            return true;
        case K_ELLIPSOID: c = zero3<T>(); r = o_max(o_max(q[0], q[1]), q[2]); return true;
        case K_OCTAHEDRON: c = zero3<T>(); r = q[0]; return true;
        case K_HEX_PRISM: c = zero3<T>(); r = o_sqrt(q[0] * q[0] + q[1] * q[1]); return true;
        case K_PLANE: return false;
        case K_CSG: return csg_bound(s.csg_nodes, s.csg_roots[o.id], c, r);
        case K_VOLUME: {
            if (s.volumes.empty()) return false;
            V3<T> lo, hi;
            s.volumes[o.id % s.volumes.size()].bounds(lo, hi);
            c = scale(lo + hi, OL(0.5));
            r = length(scale(hi - lo, OL(0.5)));
            return true;
        }
        default: return false;
    }
}

// Object::local_point (lib.rs:400-419)
template <class T> inline V3<T> local_point(const Object<T>& o, V3<T> p) {
    V3<T> l = to_local(o.xf, p);
    if (o.any_mirror()) l = op_mirror(l, o.mx, o.my, o.mz);
    if (!is_zero(o.elongate)) l = op_elongate(l, o.elongate);
    if (!is_zero(o.repeat)) l = op_repeat(l, o.repeat);
    if (o.twist != T(0)) l = op_twist(l, o.twist);
    if (o.bend != T(0)) l = op_bend(l, o.bend);
    return l;
}

// Object::field (lib.rs:380-397)
template <class T> inline Field<T> object_field(const Scene<T>& s, const Object<T>& o, V3<T> p) {
    V3<T> l = local_point(o, p);
    T d = object_prim_distance(s, o, l) * o.xf.scale;
    if (o.round != T(0)) d = op_round(d, o.round);
    if (o.onion != T(0)) d = op_onion(d, o.onion);
    return Field<T>{d, o.mat};
}

// Object::world_bound (lib.rs:470-496)
template <class T> inline bool world_bound(const Scene<T>& s, const Object<T>& o, V3<T>& wc, T& wr) {
    V3<T> center;
    T radius;
    if (!prim_local_bound(s, o, center, radius)) return false;
    if (!is_zero(o.repeat) || o.bend != T(0)) return false;
    if (o.any_mirror()) {
        radius = radius + length(center);
        center = zero3<T>();
    }
    if (o.twist != T(0)) {
        radius = radius + o_sqrt(center.x * center.x + center.z * center.z);
        center.x = T(0);
        center.z = T(0);
    }
    radius = radius + length(o.elongate);
    wc = o.xf.pos + mul_vec(o.xf.rot, scale(center, o.xf.scale));
    wr = radius * o.xf.scale + o_max(o.round, T(0)) + o_abs(o.onion);
    return true;
}

// Object::is_dual_safe (lib.rs:426-430)
template <class T> inline bool object_dual_safe(const Object<T>& o) {
    return o.twist == T(0) && o.bend == T(0) && o.prim != K_VOLUME && o.prim != K_CSG && o.prim != K_SURFACE;
}
template <class T> inline bool scene_dual_safe(const Scene<T>& s) {
    for (const auto& o : s.objects)
        if (!object_dual_safe(o)) return false;
    return true;
}

// Prim::distance_dual (lib.rs:244-261)
template <class T> inline Dual<T> prim_distance_dual(const Object<T>& o, Dual<T> x, Dual<T> y, Dual<T> z) {
    const T* q = o.p;
    switch (o.prim) {
        case K_SPHERE: return dd_sphere(x, y, z, q[0]);
        case K_BOX: return dd_box(x, y, z, V3<T>{q[0], q[1], q[2]});
        case K_ROUND_BOX: return dd_round_box(x, y, z, V3<T>{q[0], q[1], q[2]}, q[3]);
        case K_TORUS: return dd_torus(x, y, z, q[0], q[1]);
        case K_CYLINDER: return dd_cylinder(x, y, z, q[0], q[1]);
        case K_CAPSULE: return dd_capsule(x, y, z, V3<T>{q[0], q[1], q[2]}, V3<T>{q[3], q[4], q[5]}, q[6]);
        case K_CONE: return dd_round_cone(x, y, z, q[0], q[1], q[2]);
        case K_ELLIPSOID: return dd_ellipsoid(x, y, z, V3<T>{q[0], q[1], q[2]});
        case K_OCTAHEDRON: return dd_octahedron(x, y, z, q[0]);
        case K_HEX_PRISM: return dd_hex_prism(x, y, z, q[0], q[1]);
        case K_PLANE: return dd_plane(x, y, z, V3<T>{q[0], q[1], q[2]}, q[3]);
        default: return dcon(o_inf<T>());
    }
}

// Object::field_dual (lib.rs:435-463)
template <class T> inline Dual<T> object_field_dual(const Object<T>& o, Dual<T> wx, Dual<T> wy, Dual<T> wz) {
    const Xform<T>& xf = o.xf;
    T inv = o_abs(xf.scale) > OL(1e-12) ? T(1) / xf.scale : T(0);
    Dual<T> tx = dadds(wx, -xf.pos.x), ty = dadds(wy, -xf.pos.y), tz = dadds(wz, -xf.pos.z);
    M3<T> rt = transpose(xf.rot);
    Dual<T> lx = dscale(dadd(dadd(dscale(tx, rt.c[0].x), dscale(ty, rt.c[1].x)), dscale(tz, rt.c[2].x)), inv);
    Dual<T> ly = dscale(dadd(dadd(dscale(tx, rt.c[0].y), dscale(ty, rt.c[1].y)), dscale(tz, rt.c[2].y)), inv);
    Dual<T> lz = dscale(dadd(dadd(dscale(tx, rt.c[0].z), dscale(ty, rt.c[1].z)), dscale(tz, rt.c[2].z)), inv);
    if (o.any_mirror()) {
        if (o.mx) lx = dabs(lx);
        if (o.my) ly = dabs(ly);
        if (o.mz) lz = dabs(lz);
    }
    if (!is_zero(o.elongate)) dd_elongate(lx, ly, lz, o.elongate);
    if (!is_zero(o.repeat)) {
        lx = dd_rep_axis(lx, o.repeat.x);
        ly = dd_rep_axis(ly, o.repeat.y);
        lz = dd_rep_axis(lz, o.repeat.z);
    }
    Dual<T> d = dscale(prim_distance_dual(o, lx, ly, lz), xf.scale);
    if (o.round != T(0)) d = dadds(d, -o.round);
    if (o.onion != T(0)) d = dadds(dabs(d), -o.onion);
    return d;
}

// Scene::normal_dual (lib.rs:820-835): exact gradient, every object, no pruning.
template <class T> inline V3<T> normal_dual(const Scene<T>& s, V3<T> p) {
    Hooks<T>::dual_eval();
    Dual<T> x{p.x, V3<T>{T(1), T(0), T(0)}}, y{p.y, V3<T>{T(0), T(1), T(0)}}, z{p.z, V3<T>{T(0), T(0), T(1)}};
    bool have = false;
    Dual<T> acc{};
    for (const auto& o : s.objects) {
        Dual<T> f = object_field_dual(o, x, y, z);
        if (!have) {
            acc = f;
            have = true;
            continue;
        }
        if (o.combine == MM3E_COMBINE_UNION) acc = dd_union(acc, f);
        else if (o.combine == MM3E_COMBINE_SMOOTH) acc = dd_smooth_union(acc, f, o.k);
        else acc = dd_subtract(acc, f);
    }
    if (!have) return zero3<T>();
    return normalize(acc.g);
}

// ------------------------------------------------------------------------------------------
// accel.rs — WorldPlan: BVH over plain-union runs
// ------------------------------------------------------------------------------------------
template <class T> struct BvhNode {
    V3<T> center;
    T radius;
    uint32_t left, right;
    int32_t leaf;
};

template <class T> struct Bvh {
    std::vector<BvhNode<T>> nodes;
    uint32_t root = 0;
};

// accel.rs:26-36
template <class T> inline void bvh_enclose(V3<T> c1, T r1, V3<T> c2, T r2, V3<T>& c, T& r) {
    T d = length(c2 - c1);
    if (d + r2 <= r1) { c = c1; r = r1; return; }
    if (d + r1 <= r2) { c = c2; r = r2; return; }
    T radius = (d + r1 + r2) * OL(0.5);
    c = c1 + scale(c2 - c1, (radius - r1) / o_max(d, OL(1e-12)));
    r = radius;
}

template <class T> struct BvhItem {
    uint64_t index;
    V3<T> c;
    T r;
};

// accel.rs:39-77  median split on the longest centroid axis, ties by index
template <class T> inline uint32_t bvh_build(BvhItem<T>* items, size_t n, std::vector<BvhNode<T>>& nodes) {
    if (n == 1) {
        nodes.push_back(BvhNode<T>{items[0].c, items[0].r, 0, 0, (int32_t)items[0].index});
        return (uint32_t)(nodes.size() - 1);
    }
    V3<T> lo = splat(o_inf<T>()), hi = splat(-o_inf<T>());
    for (size_t i = 0; i < n; ++i) {
        lo = vmin(lo, items[i].c);
        hi = vmax(hi, items[i].c);
    }
    V3<T> ext = hi - lo;
    int axis = (ext.x >= ext.y && ext.x >= ext.z) ? 0 : (ext.y >= ext.z ? 1 : 2);
    auto coord = [axis](const V3<T>& c) { return axis == 0 ? c.x : (axis == 1 ? c.y : c.z); };
    std::sort(items, items + n, [&](const BvhItem<T>& a, const BvhItem<T>& b) {
        double ca = o_value(coord(a.c)), cb = o_value(coord(b.c));
        if (ca < cb) return true;
        if (ca > cb) return false;
        return a.index < b.index;
    });
    size_t mid = n / 2;
    uint32_t left = bvh_build(items, mid, nodes);
    uint32_t right = bvh_build(items + mid, n - mid, nodes);
    V3<T> c;
    T r;
    bvh_enclose(nodes[left].center, nodes[left].radius, nodes[right].center, nodes[right].radius, c, r);
    nodes.push_back(BvhNode<T>{c, r, left, right, -1});
    return (uint32_t)(nodes.size() - 1);
}

template <class T> struct Segment {
    bool one = false;
    uint64_t index = 0;            // Segment::One
    std::optional<Bvh<T>> tree;    // Segment::Run
    std::vector<uint64_t> unbounded;
};

template <class T> struct Best {
    T dist;
    int64_t index;
    uint32_t mat;
};

template <class T> struct WorldPlan {
    std::vector<Segment<T>> segments;
    std::vector<bool> has_bound;
    std::vector<V3<T>> bound_c;
    std::vector<T> bound_r;
    T slack = T(0);

    // accel.rs:134-185
    void build(const Scene<T>& s) {
        size_t n = s.objects.size();
        has_bound.assign(n, false);
        bound_c.assign(n, zero3<T>());
        bound_r.assign(n, T(0));
        T mk = T(0);
        for (size_t i = 0; i < n; ++i) {
            has_bound[i] = world_bound(s, s.objects[i], bound_c[i], bound_r[i]);
            T k = s.objects[i].combine == MM3E_COMBINE_SMOOTH ? s.objects[i].k : T(0);
            mk = o_max(mk, k);
        }
        slack = mk + OL(0.1);
        std::vector<uint64_t> run;
        auto close_run = [&]() {
            if (run.empty()) return;
            std::vector<BvhItem<T>> items;
            Segment<T> seg;
            for (uint64_t i : run) {
                if (has_bound[i]) items.push_back(BvhItem<T>{i, bound_c[i], bound_r[i]});
                else seg.unbounded.push_back(i);
            }
            if (!items.empty()) {
                Bvh<T> b;
                b.nodes.reserve(items.size() * 2);
                b.root = bvh_build(items.data(), items.size(), b.nodes);
                seg.tree = std::move(b);
            }
            segments.push_back(std::move(seg));
            run.clear();
        };
        for (size_t i = 0; i < n; ++i) {
            if (s.objects[i].combine == MM3E_COMBINE_UNION) {
                run.push_back(i);
            } else {
                close_run();
                Segment<T> seg;
                seg.one = true;
                seg.index = i;
                segments.push_back(std::move(seg));
            }
        }
        close_run();
    }

    // accel.rs:187-207
    Field<T> contrib(const Scene<T>& s, uint64_t i, V3<T> p) const {
        if (has_bound[i]) {
            T lower = length(p - bound_c[i]) - bound_r[i];
            if (lower > slack) return Field<T>{lower, s.objects[i].mat};
        }
        return object_field(s, s.objects[i], p);
    }

    // accel.rs:79-119
    void query(const Scene<T>& s, const Bvh<T>& b, V3<T> p, Best<T>& best) const {
        uint32_t stack[64];
        size_t sp = 0;
        stack[sp++] = b.root;
        while (sp > 0) {
            const BvhNode<T>& node = b.nodes[stack[--sp]];
            T lower = length(p - node.center) - node.radius;
            if (lower > best.dist) continue;
            if (node.leaf >= 0) {
                uint64_t i = (uint64_t)node.leaf;
                Field<T> c = lower > slack ? Field<T>{lower, s.objects[i].mat} : object_field(s, s.objects[i], p);
                if (c.dist < best.dist || (c.dist == best.dist && (int64_t)i < best.index)) best = Best<T>{c.dist, (int64_t)i, c.mat};
            } else {
                T ld = length_sq(p - b.nodes[node.left].center);
                T rd = length_sq(p - b.nodes[node.right].center);
                uint32_t nearn = ld <= rd ? node.left : node.right;
                uint32_t farn = ld <= rd ? node.right : node.left;
                stack[sp] = farn;
                stack[sp + 1] = nearn;
                sp += 2;
            }
        }
    }

    // accel.rs:209-252
    Field<T> eval(const Scene<T>& s, V3<T> p) const {
        Field<T> acc = field_far<T>();
        bool seeded = false;
        for (const auto& seg : segments) {
            if (seg.one) {
                Field<T> f = contrib(s, seg.index, p);
                if (!seeded) {
                    acc = f;
                    seeded = true;
                    continue;
                }
                const Object<T>& o = s.objects[seg.index];
                if (o.combine == MM3E_COMBINE_UNION) acc = f_union(acc, f);
                else if (o.combine == MM3E_COMBINE_SMOOTH) acc = f_smooth_union(acc, f, o.k);
                else acc = f_subtract(acc, f);
            } else {
                Best<T> best = seeded ? Best<T>{acc.dist, -1, acc.mat} : Best<T>{o_inf<T>(), INT64_MAX, 0u};
                for (uint64_t i : seg.unbounded) {
                    Field<T> f = object_field(s, s.objects[i], p);
                    if (f.dist < best.dist || (f.dist == best.dist && (int64_t)i < best.index)) best = Best<T>{f.dist, (int64_t)i, f.mat};
                }
                if (seg.tree) query(s, *seg.tree, p, best);
                acc = Field<T>{best.dist, best.mat};
                seeded = true;
            }
        }
        return acc;
    }
};

// The world field closure (lib.rs:758-761), with the linear reference fold (lib.rs:766-807).
template <class T> struct World {
    const Scene<T>* s;
    WorldPlan<T> plan;
    explicit World(const Scene<T>& sc) : s(&sc) { plan.build(sc); }
    Field<T> operator()(V3<T> p) const {
        Hooks<T>::field_eval();
        return plan.eval(*s, p);
    }
    // lib.rs:766-807
    Field<T> linear(V3<T> p) const {
        Field<T> acc = field_far<T>();
        bool first = true;
        for (size_t i = 0; i < s->objects.size(); ++i) {
            const Object<T>& o = s->objects[i];
            Field<T> f = plan.has_bound[i] && (length(p - plan.bound_c[i]) - plan.bound_r[i]) > plan.slack
                             ? Field<T>{length(p - plan.bound_c[i]) - plan.bound_r[i], o.mat}
                             : object_field(*s, o, p);
            if (first) {
                first = false;
                acc = f;
                continue;
            }
            if (o.combine == MM3E_COMBINE_UNION) acc = f_union(acc, f);
            else if (o.combine == MM3E_COMBINE_SMOOTH) acc = f_smooth_union(acc, f, o.k);
            else acc = f_subtract(acc, f);
        }
        return acc;
    }
};

// ------------------------------------------------------------------------------------------
// lib.rs render path
// ------------------------------------------------------------------------------------------
template <class T>
inline Hit<T> march_scene(const Scene<T>& s, const World<T>& w, bool dual_safe, const Ray<T>& ray, uint32_t depth = 0) {
    PhaseScope<T> ph(depth == 0 ? PH_MARCH : PH_MARCH_REFL);
    if (dual_safe) return s.marcher.march_with(w, [&](V3<T> p) { return normal_dual(s, p); }, ray);
    return s.marcher.march_with(w, [&](V3<T> p) { return s.marcher.normal(w, p); }, ray);
}

// lib.rs:1365-1375
template <class T> inline V3<T> surface_albedo(const Material<T>& m, V3<T> p) {
    if (!m.checker) return m.albedo;
    int32_t ix = o_to_i32(o_floor(p.x));
    int32_t iz = o_to_i32(o_floor(p.z));
    int32_t sum = (int32_t)((uint32_t)ix + (uint32_t)iz);
    int32_t rem = sum % 2;
    if (rem < 0) rem += 2;
    bool parity = rem == 0;
    V3<T> base = parity ? splat(OL(0.92)) : splat(OL(0.20));
    T tint = T(hash_cell(ix, iz)) * OL(0.06) - OL(0.03);
    return max_scalar(cmul(base + splat(tint), m.albedo), T(0));
}

// appearance.rs:427-432 (no UV bindings: material % len + checker albedo)
template <class T> inline Material<T> material_for_hit(const Scene<T>& s, const Hit<T>& h) {
    Material<T> m = s.materials[h.mat % s.materials.size()];
    m.albedo = surface_albedo(m, h.pos);
    return m;
}

// lib.rs:1379-1398
template <class T> inline V3<T> ibl_irradiance(const Scene<T>& s, V3<T> n) {
    V3<T> up = o_abs(n.y) > OL(0.9) ? V3<T>{T(1), T(0), T(0)} : V3<T>{T(0), T(1), T(0)};
    V3<T> t1 = normalize(cross(n, up));
    V3<T> t2 = normalize(cross(n, t1));
    V3<T> n6 = scale(n, OL(0.6));
    V3<T> dirs[5] = {n, normalize(n6 + scale(t1, OL(0.6))), normalize(n6 - scale(t1, OL(0.6))),
                     normalize(n6 + scale(t2, OL(0.6))), normalize(n6 - scale(t2, OL(0.6)))};
    V3<T> acc = zero3<T>();
    T w = T(0);
    for (int i = 0; i < 5; ++i) {
        T cw = o_max(dot(dirs[i], n), T(0));
        acc = acc + scale(sky_diffuse(dirs[i], s.sun_dir), cw);
        w = w + cw;
    }
    return cmul(scale(acc, T(1) / o_max(w, OL(1e-4))), s.sky_ambient);
}

// lib.rs:1401-1407
template <class T> inline V3<T> heatmap(T t) {
    t = o_clamp(t, T(0), T(1));
    T r = o_clamp(t * T(3) - OL(1.5), T(0), T(1));
    T g = o_clamp(T(1) - o_abs(t * T(3) - OL(1.3)), T(0), T(1));
    T b = o_clamp(T(1) - t * OL(2.2), T(0), T(1));
    return V3<T>{r, g, b};
}

template <class T> V3<T> trace(const Scene<T>& s, const World<T>& w, const Ray<T>& ray, uint32_t depth, bool dual_safe);

// lib.rs:1286-1360
template <class T>
inline V3<T> shade_hit(const Scene<T>& s, const World<T>& w, const Hit<T>& hit, const Ray<T>& ray, uint32_t depth, bool dual_safe) {
    Material<T> m = material_for_hit(s, hit);
    V3<T> albedo = m.albedo;
    V3<T> normal = hit.normal;
    V3<T> view = scale(ray.dir, T(-1));
    T occ = T(1);
    if (s.ao) {
        PhaseScope<T> ph(depth == 0 ? PH_AO : PH_AO_REFL);
        occ = s.marcher.ambient_occlusion(w, hit.pos, hit.normal);
    }
    V3<T> gi = s.gi ? s.gi->sample(hit.pos, normal) : zero3<T>();
    V3<T> ambient_irr = ibl_irradiance(s, normal) + gi + s.ambient;
    V3<T> radiance = scale(cmul(albedo, ambient_irr), occ);
    for (const auto& light : s.lights) {
        V3<T> l_dir;
        T l_dist;
        light.toward(hit.pos, l_dir, l_dist);
        if (lambert(normal, l_dir) <= T(0)) continue;
        T shadow = T(1);
        if (s.shadows) {
            T max_t = o_min(l_dist, s.marcher.max_dist);
            T lift = o_max(s.marcher.normal_h * T(2), OL(0.01));
            Hooks<T>::shadow_ray();
            PhaseScope<T> ph(depth == 0 ? PH_SHADOW : PH_SHADOW_REFL);
            shadow = s.marcher.soft_shadow(w, hit.pos + scale(hit.normal, lift), l_dir, max_t, light.shadow_k(l_dist));
        }
        if (shadow <= T(0)) continue;
        V3<T> surface = brdf(normal, l_dir, view, albedo, m.metallic, m.roughness, m.specular);
        radiance = radiance + scale(cmul(surface, light.color), shadow * light.attenuation(l_dist));
    }
    if (depth < s.bounces && m.reflectivity > T(0)) {
        T cosv = o_max(dot(normal, view), T(0));
        T fr = fresnel_schlick(cosv, m.reflectivity);
        V3<T> rdir = normalize(reflect(ray.dir, normal));
        V3<T> rorigin = hit.pos + scale(hit.normal, o_max(s.marcher.normal_h * T(2), OL(0.02)));
        V3<T> refl = trace(s, w, Ray<T>{rorigin, rdir}, depth + 1, dual_safe);
        radiance = scale(radiance, T(1) - fr) + scale(refl, fr);
    }
    radiance = radiance + m.emissive;
    return apply_fog(radiance, s.fog, hit.t, s.fog_density);
}

// ------------------------------------------------------------------------------------------
// film.rs — render_film samples (thin lens, coverage, premultiplied foreground)
// ------------------------------------------------------------------------------------------
// film.rs:218-224
inline uint32_t film_hash(uint32_t v) {
    v ^= v >> 16;
    v *= 0x7feb352du;
    v ^= v >> 15;
    v *= 0x846ca68bu;
    return v ^ (v >> 16);
}

// film.rs:199-215: one jittered sample per aperture grid cell, pixel-dependent shifts.
template <class T> inline void aperture_sample(uint32_t px, uint32_t py, uint32_t sx, uint32_t sy, uint32_t n, T& u,
                                               T& v) {
    if (n == 1) {
        u = OL(0.5);
        v = OL(0.5);
        return;
    }
    uint32_t pixel_seed = film_hash(px ^ film_hash(py));
    uint64_t n64 = n;
    uint32_t cell_x = (uint32_t)(((uint64_t)sx + sy + pixel_seed) % n64);
    uint32_t cell_y = (uint32_t)(((uint64_t)sx + 2ull * sy + film_hash(pixel_seed)) % n64);
    uint32_t seed = film_hash(pixel_seed ^ film_hash(sx) ^ film_hash(sy + 0xa511e9b3u));
    auto unit = [](uint32_t value) { return T((float)(value >> 8)) * OL(1.0 / 16777216.0); };
    u = (T((float)cell_x) + unit(seed)) / T((float)n);
    v = (T((float)cell_y) + unit(film_hash(seed))) / T((float)n);
}

// camera.rs:92-102: equal-area concentric square-to-disk map.
template <class T> inline void concentric_disk(T s0, T s1, T& dx, T& dy) {
    T x = T(2) * s0 - T(1);
    T y = T(2) * s1 - T(1);
    if (x == T(0) && y == T(0)) {
        dx = T(0);
        dy = T(0);
        return;
    }
    T radius, theta;
    if (o_abs(x) > o_abs(y)) {
        radius = x;
        theta = OL(0.785398163397448309616) * (y / x);
    } else {
        radius = y;
        theta = OL(1.57079632679489661923) - OL(0.785398163397448309616) * (x / y);
    }
    dx = radius * o_cos(theta);
    dy = radius * o_sin(theta);
}

// camera.rs:71-90: thin-lens ray through a fractional image sample.
template <class T>
inline Ray<T> camera_ray_lens(const Camera<T>& c, T ix, T iy, uint32_t w, uint32_t h, T radius, T focus, T a0, T a1) {
    Ray<T> pinhole = camera_ray(c, ix, iy, w, h);
    if (radius == T(0)) return pinhole;
    T dx, dy;
    concentric_disk(a0, a1, dx, dy);
    V3<T> origin = c.eye + scale(c.right, dx * radius) + scale(c.up, dy * radius);
    V3<T> fp = c.eye + scale(pinhole.dir, focus / dot(pinhole.dir, c.forward));
    return Ray<T>{origin, normalize(fp - origin)};
}

template <class T> struct FilmSample {
    V3<T> beauty, foreground;
    T alpha;
    Hit<T> center;
};

// film.rs:147-196 (sample_pixel)
template <class T>
inline FilmSample<T> film_sample_pixel(const Scene<T>& s, const World<T>& w, const Camera<T>& cam, T radius, T focus,
                                       uint32_t x, uint32_t y, bool dual_safe) {
    Ray<T> center_ray = camera_ray(cam, T((float)x) + OL(0.5), T((float)y) + OL(0.5), s.width, s.height);
    Hit<T> center = march_scene(s, w, dual_safe, center_ray, 0);
    uint32_t n = s.aa > 1 ? s.aa : 1;
    T inv_samples = T(1) / T((float)((uint64_t)n * n));
    V3<T> beauty = zero3<T>(), fg = zero3<T>();
    uint64_t hits = 0;
    for (uint32_t sy = 0; sy < n; ++sy)
        for (uint32_t sx = 0; sx < n; ++sx) {
            T ix = T((float)x) + (T((float)sx) + OL(0.5)) / T((float)n);
            T iy = T((float)y) + (T((float)sy) + OL(0.5)) / T((float)n);
            T a0, a1;
            aperture_sample(x, y, sx, sy, n, a0, a1);
            Ray<T> ray = n == 1 ? center_ray : camera_ray_lens(cam, ix, iy, s.width, s.height, radius, focus, a0, a1);
            Hit<T> hit = n == 1 ? center : march_scene(s, w, dual_safe, ray, 0);
            if (hit.hit) {
                V3<T> rad = shade_hit(s, w, hit, ray, 0, dual_safe);
                beauty = beauty + rad;
                fg = fg + rad;
                hits += 1;
            } else {
                beauty = beauty + sky(ray.dir, s.sun_dir);
            }
        }
    return FilmSample<T>{scale(beauty, inv_samples), scale(fg, inv_samples), T((float)hits) * inv_samples, center};
}

// lib.rs:1265-1282
template <class T> V3<T> trace(const Scene<T>& s, const World<T>& w, const Ray<T>& ray, uint32_t depth, bool dual_safe) {
    if (depth == 0) Hooks<T>::primary_ray();
    else Hooks<T>::reflection_ray();
    Hit<T> hit = march_scene(s, w, dual_safe, ray, depth);
    if (!hit.hit) return sky(ray.dir, s.sun_dir);
    return shade_hit(s, w, hit, ray, depth, dual_safe);
}

// lib.rs:1223-1243
template <class T>
inline V3<T> shade_pixel(const Scene<T>& s, const World<T>& w, const Camera<T>& cam, uint32_t x, uint32_t y, bool dual_safe) {
    uint32_t n = s.aa > 1 ? s.aa : 1;
    T nf = T((float)n);
    T inv_samples = T(1) / T((float)(n * n));
    V3<T> acc = zero3<T>();
    for (uint32_t sy = 0; sy < n; ++sy) {
        for (uint32_t sx = 0; sx < n; ++sx) {
            T ox = (T((float)sx) + OL(0.5)) / nf;
            T oy = (T((float)sy) + OL(0.5)) / nf;
            Ray<T> ray = camera_ray(cam, T((float)x) + ox, T((float)y) + oy, s.width, s.height);
            acc = acc + trace(s, w, ray, 0, dual_safe);
        }
    }
    return scale(acc, inv_samples);
}

// lib.rs:1178-1218  debug AOV pixel (no post)
template <class T>
inline V3<T> aov_pixel(const Scene<T>& s, const World<T>& w, const Camera<T>& cam, uint32_t x, uint32_t y, bool dual_safe) {
    Ray<T> ray = camera_ray(cam, T((float)x) + OL(0.5), T((float)y) + OL(0.5), s.width, s.height);
    Hit<T> hit = march_scene(s, w, dual_safe, ray);
    switch (s.mode) {
        case MM3E_MODE_NORMAL:
            return hit.hit ? scale(hit.normal, OL(0.5)) + splat(OL(0.5)) : zero3<T>();
        case MM3E_MODE_DEPTH: {
            T d = o_clamp(hit.t / s.marcher.max_dist, T(0), T(1));
            return splat(T(1) - d);
        }
        case MM3E_MODE_AO:
            return hit.hit ? splat(s.marcher.ambient_occlusion(w, hit.pos, hit.normal)) : one3<T>();
        case MM3E_MODE_STEPS:
            return heatmap(T((float)hit.steps) / T((float)s.marcher.max_steps));
        case MM3E_MODE_ALBEDO:
            return hit.hit ? material_for_hit(s, hit).albedo : zero3<T>();
        default:
            return zero3<T>();
    }
}

// Row bands exactly as render_linear_unchecked / render_bands_with_threads (lib.rs:908-947,
// 1135-1175): threads.max(1).min(h); the first h % threads bands take one extra row.
template <class F> inline void for_row_bands(uint32_t y0, uint32_t y1, unsigned threads, F&& body) {
    uint32_t h = y1 > y0 ? y1 - y0 : 0;
    if (h == 0) return;
    size_t t = threads > 0 ? threads : 1;
    if (t > h) t = h;
    size_t band = h / t, extra = h % t;
    std::vector<std::thread> pool;
    for (size_t ti = 0; ti < t; ++ti) {
        uint32_t a = y0 + (uint32_t)(ti * band + std::min(ti, extra));
        uint32_t b = a + (uint32_t)band + (ti < extra ? 1u : 0u);
        pool.emplace_back([&body, a, b, ti]() { body(a, b, ti); });
    }
    for (auto& th : pool) th.join();
}

// Beauty radiance for rows [y0, y1) (render_linear_unchecked).
template <class T>
inline void render_linear_rows(const Scene<T>& s, const Camera<T>& cam, uint32_t y0, uint32_t y1, unsigned threads, V3<T>* out_rows) {
    bool dual_safe = scene_dual_safe(s);
    for_row_bands(y0, y1, threads, [&](uint32_t a, uint32_t b, size_t) {
        World<T> w(s);  // one world plan per band, as the reference builds per worker
        for (uint32_t y = a; y < b; ++y)
            for (uint32_t x = 0; x < s.width; ++x)
                out_rows[(size_t)(y - y0) * s.width + x] = shade_pixel(s, w, cam, x, y, dual_safe);
    });
}

// post.rs:331-345
template <class T> inline std::vector<T> gaussian_kernel(uint32_t radius) {
    int32_t r = (int32_t)(radius > 1 ? radius : 1);
    T sigma = o_max(T((float)r) / T(2), OL(1e-3));
    std::vector<T> k;
    T sum = T(0);
    for (int32_t i = -r; i <= r; ++i) {
        T v = o_exp(T((float)(-(i * i))) / (T(2) * sigma * sigma));
        k.push_back(v);
        sum = sum + v;
    }
    for (auto& v : k) v = v / sum;
    return k;
}

// post.rs:348-368
template <class T>
inline std::vector<V3<T>> blur_axis(const std::vector<V3<T>>& src, uint32_t w, uint32_t h, const std::vector<T>& kernel, bool horizontal) {
    std::vector<V3<T>> out(src.size(), zero3<T>());
    if (w == 0 || h == 0) return out;
    int32_t r = (int32_t)(kernel.size() / 2);
    int32_t wi = (int32_t)w, hi = (int32_t)h;
    for (int32_t y = 0; y < hi; ++y) {
        for (int32_t x = 0; x < wi; ++x) {
            V3<T> acc = zero3<T>();
            for (size_t ki = 0; ki < kernel.size(); ++ki) {
                int32_t off = (int32_t)ki - r;
                int32_t sx = horizontal ? std::clamp(x + off, 0, wi - 1) : x;
                int32_t sy = horizontal ? y : std::clamp(y + off, 0, hi - 1);
                acc = acc + scale(src[(size_t)sy * w + sx], kernel[ki]);
            }
            out[(size_t)y * w + x] = acc;
        }
    }
    return out;
}

// post.rs:36-58 (+ bloom_pass post.rs:61-75): HDR -> RGBA f32 framebuffer (alpha 1).
template <class T> inline void post_resolve(const std::vector<V3<T>>& hdr, uint32_t w, uint32_t h, const Post<T>& post, float* rgba) {
    size_t n = (size_t)w * h;
    std::vector<V3<T>> color(hdr.begin(), hdr.begin() + n);
    if (post.bloom && post.intensity > T(0)) {
        std::vector<V3<T>> bright(n, zero3<T>());
        for (size_t i = 0; i < n; ++i) {
            T l = luminance(color[i]);
            if (l > post.threshold) bright[i] = scale(color[i], (l - post.threshold) / o_max(l, OL(1e-4)));
        }
        std::vector<T> kernel = gaussian_kernel<T>(post.radius);
        std::vector<V3<T>> horiz = blur_axis(bright, w, h, kernel, true);
        std::vector<V3<T>> bloom = blur_axis(horiz, w, h, kernel, false);
        for (size_t i = 0; i < n; ++i) color[i] = color[i] + scale(bloom[i], post.intensity);
    }
    for (size_t i = 0; i < n; ++i) {
        V3<T> c = clamp01(gamma(aces(scale(color[i], post.exposure))));
        rgba[4 * i + 0] = (float)o_value(c.x);
        rgba[4 * i + 1] = (float)o_value(c.y);
        rgba[4 * i + 2] = (float)o_value(c.z);
        rgba[4 * i + 3] = 1.0f;
    }
}

// Full frame: render_unchecked (lib.rs:872-883) -> RGBA f32 framebuffer.
template <class T>
inline void render_frame(const Scene<T>& s, const Camera<T>& cam, unsigned threads, float* rgba, V3<T>* hdr_out) {
    uint32_t w = s.width, h = s.height;
    size_t n = (size_t)w * h;
    if (n == 0) return;
    if (s.mode != MM3E_MODE_BEAUTY) {
        bool dual_safe = scene_dual_safe(s);
        for_row_bands(0, h, threads, [&](uint32_t a, uint32_t b, size_t) {
            World<T> wd(s);
            for (uint32_t y = a; y < b; ++y)
                for (uint32_t x = 0; x < w; ++x) {
                    V3<T> v = clamp01(aov_pixel(s, wd, cam, x, y, dual_safe));
                    size_t i = (size_t)y * w + x;
                    rgba[4 * i + 0] = (float)o_value(v.x);
                    rgba[4 * i + 1] = (float)o_value(v.y);
                    rgba[4 * i + 2] = (float)o_value(v.z);
                    rgba[4 * i + 3] = 1.0f;
                }
        });
        return;
    }
    std::vector<V3<T>> hdr(n);
    render_linear_rows(s, cam, 0, h, threads, hdr.data());
    if (hdr_out)
        for (size_t i = 0; i < n; ++i) hdr_out[i] = hdr[i];
    post_resolve(hdr, w, h, s.post, rgba);
}

// ------------------------------------------------------------------------------------------
// gi.rs + Scene::bake_gi_unchecked / gather (lib.rs:668-711)
// ------------------------------------------------------------------------------------------
// gi.rs:38-50
template <class T> inline std::vector<std::pair<V3<T>, T>> axis_dirs(V3<T> axis, uint32_t samples) {
    V3<T> up = o_abs(axis.y) > OL(0.9) ? V3<T>{T(1), T(0), T(0)} : V3<T>{T(0), T(1), T(0)};
    V3<T> t1 = normalize(cross(axis, up));
    V3<T> t2 = normalize(cross(axis, t1));
    std::vector<std::pair<V3<T>, T>> dirs{{axis, T(1)}};
    if (samples > 1) {
        V3<T> ts[4] = {t1, t2, scale(t1, T(-1)), scale(t2, T(-1))};
        for (auto& t : ts) {
            V3<T> d = normalize(scale(axis, OL(0.72)) + scale(t, OL(0.72)));
            dirs.push_back({d, o_max(dot(d, axis), T(0))});
        }
    }
    return dirs;
}

// lib.rs:686-711 one-bounce gather (no shadows)
template <class T> inline V3<T> gi_gather(const Scene<T>& s, const World<T>& w, bool dual_safe, V3<T> origin, V3<T> dir) {
    Hooks<T>::gi_ray();
    Ray<T> ray{origin, dir};
    Hit<T> hit = march_scene(s, w, dual_safe, ray);
    if (!hit.hit) return sky_diffuse(dir, s.sun_dir);
    Material<T> m = material_for_hit(s, hit);
    V3<T> n = hit.normal;
    V3<T> c = m.emissive;
    for (const auto& light : s.lights) {
        V3<T> l_dir;
        T l_dist;
        light.toward(hit.pos, l_dir, l_dist);
        T ndl = lambert(n, l_dir);
        if (ndl > T(0)) {
            V3<T> outgoing = brdf(n, l_dir, scale(dir, T(-1)), m.albedo, m.metallic, m.roughness, m.specular);
            c = c + scale(cmul(outgoing, light.color), light.attenuation(l_dist));
        }
    }
    return c;
}

// gi.rs:192-203 over Object::world_bound spheres, pad 1.5 (lib.rs:669-671)
template <class T> inline bool gi_bounds(const Scene<T>& s, V3<T>& lo, V3<T>& hi) {
    bool any = false;
    lo = splat(o_inf<T>());
    hi = splat(-o_inf<T>());
    for (const auto& o : s.objects) {
        V3<T> c;
        T r;
        if (!world_bound(s, o, c, r)) continue;
        any = true;
        lo = vmin(lo, c - splat(r));
        hi = vmax(hi, c + splat(r));
    }
    if (!any) return false;
    lo = lo - splat(OL(1.5));
    hi = hi + splat(OL(1.5));
    return true;
}

// gi.rs:55-125 with the gather above; returns false when the scene has no bounded object.
template <class T> inline bool bake_gi(const Scene<T>& s, uint64_t dx, uint64_t dy, uint64_t dz, uint32_t samples, unsigned threads, GiVolume<T>& out) {
    V3<T> lo, hi;
    if (!gi_bounds(s, lo, hi)) return false;
    uint64_t nx = dx > 1 ? dx : 1, ny = dy > 1 ? dy : 1, nz = dz > 1 ? dz : 1;
    V3<T> size = hi - lo;
    V3<T> cell{size.x / T((float)((nx > 2 ? nx : 2) - 1)), size.y / T((float)((ny > 2 ? ny : 2) - 1)),
               size.z / T((float)((nz > 2 ? nz : 2) - 1))};
    const V3<T> axes[6] = {{T(1), T(0), T(0)}, {T(-1), T(0), T(0)}, {T(0), T(1), T(0)},
                           {T(0), T(-1), T(0)}, {T(0), T(0), T(1)}, {T(0), T(0), T(-1)}};
    std::vector<std::vector<std::pair<V3<T>, T>>> dir_sets;
    for (auto& a : axes) dir_sets.push_back(axis_dirs(a, samples));
    bool dual_safe = scene_dual_safe(s);
    out.min = lo;
    out.size = size;
    out.nx = nx;
    out.ny = ny;
    out.nz = nz;
    out.cubes.assign(nx * ny * nz, std::array<V3<T>, 6>{});
    for_row_bands(0, (uint32_t)nz, threads, [&](uint32_t k0, uint32_t k1, size_t) {
        World<T> w(s);
        for (uint64_t k = k0; k < k1; ++k)
            for (uint64_t j = 0; j < ny; ++j)
                for (uint64_t i = 0; i < nx; ++i) {
                    V3<T> probe = lo + V3<T>{T((float)i) * cell.x, T((float)j) * cell.y, T((float)k) * cell.z};
                    std::array<V3<T>, 6> cube;
                    for (int a = 0; a < 6; ++a) {
                        V3<T> acc = zero3<T>();
                        T wsum = T(0);
                        for (auto& dw : dir_sets[a]) {
                            acc = acc + scale(gi_gather(s, w, dual_safe, probe, dw.first), dw.second);
                            wsum = wsum + dw.second;
                        }
                        cube[a] = scale(acc, T(1) / o_max(wsum, OL(1e-4)));
                    }
                    out.cubes[(k * ny + j) * nx + i] = cube;
                }
    });
    return true;
}

}  // namespace oracle
