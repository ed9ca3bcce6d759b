// oracle_capi.cpp — C entry points of the CPU oracle (liboracle_mm3e.so).
//
// TEST INFRASTRUCTURE ONLY. Loaded by the tests, by __graft_entry__.smoke() and by bench.py's
// CPU-baseline leg, always as the checker or the timed CPU reference — never by the product
// library. Every function takes the same `mm3e_scene_desc` / `mm3e_camera` as the C ABI.
#include <chrono>
#include <cstring>
#include <mutex>

#include "oracle_count.hpp"
#include "oracle_mesh.hpp"
#include "oracle_scene.hpp"

using namespace oracle;

namespace {

template <class T> Camera<T> cam_from(const mm3e_camera& c) {
    Camera<T> k;
    k.eye = v3f<T>(c.eye);
    k.forward = v3f<T>(c.forward);
    k.right = v3f<T>(c.right);
    k.up = v3f<T>(c.up);
    k.fov_scale = T(c.fov_scale);
    return k;
}

// Rust f32 `rem_euclid` (core::f32::rem_euclid).
float rem_euclid_f32(float a, float b) {
    float r = std::fmod(a, b);
    return r < 0.0f ? r + std::fabs(b) : r;
}

// vec.rs:136-141 Rodrigues
M3<float> from_axis_angle(V3<float> axis, float angle) {
    V3<float> k = normalize(axis);
    float s = o_sin(angle), c = o_cos(angle);
    auto col = [&](V3<float> e) { return scale(e, c) + scale(cross(k, e), s) + scale(k, dot(k, e) * (1.0f - c)); };
    M3<float> m;
    m.c[0] = col(V3<float>{1, 0, 0});
    m.c[1] = col(V3<float>{0, 1, 0});
    m.c[2] = col(V3<float>{0, 0, 1});
    return m;
}
M3<float> mat_mul(const M3<float>& a, const M3<float>& b) {
    M3<float> r;
    for (int i = 0; i < 3; ++i) r.c[i] = mul_vec(a, b.c[i]);
    return r;
}

}  // namespace

extern "C" {

int oracle_abi_version(void) { return MM3E_ABI_VERSION; }

// Camera::look_at (camera.rs:50-55)
void oracle_camera_look_at(const float eye[3], const float target[3], const float up[3], float fov_y, mm3e_camera* out) {
    Camera<float> c = camera_look_at(v3f<float>(eye), v3f<float>(target), v3f<float>(up), fov_y);
    const V3<float>* vs[4] = {&c.eye, &c.forward, &c.right, &c.up};
    float* dst[4] = {out->eye, out->forward, out->right, out->up};
    for (int i = 0; i < 4; ++i) {
        dst[i][0] = vs[i]->x;
        dst[i][1] = vs[i]->y;
        dst[i][2] = vs[i]->z;
    }
    out->fov_scale = c.fov_scale;
}

// orbit_camera + wrap_orbit_yaw (mm3e-orchestrator/src/lib.rs:1414-1435)
void oracle_orbit_camera(const float target[3], float radius, float yaw, float pitch, float fov_y, mm3e_camera* out) {
    const float PI = 3.14159265358979323846f, TAU = 6.28318530717958647692f, FRAC_PI_2 = 1.57079632679489661923f;
    yaw = std::isfinite(yaw) ? rem_euclid_f32(yaw + PI, TAU) - PI : 0.0f;
    float pitch_limit = FRAC_PI_2 - 1.0e-4f;
    pitch = std::isfinite(pitch) ? o_clamp(pitch, -pitch_limit, pitch_limit) : 0.0f;
    radius = std::isfinite(radius) ? o_max(std::fabs(radius), 1.0e-4f) : 1.0f;
    fov_y = std::isfinite(fov_y) ? o_clamp(fov_y, 1.0e-4f, PI - 1.0e-4f) : 45.0f * (PI / 180.0f);
    V3<float> t = v3f<float>(target);
    V3<float> eye = t + V3<float>{radius * o_cos(yaw) * o_cos(pitch), radius * o_sin(pitch), radius * o_sin(yaw) * o_cos(pitch)};
    float e[3] = {eye.x, eye.y, eye.z};
    float up[3] = {0.0f, 1.0f, 0.0f};
    oracle_camera_look_at(e, target, up, fov_y, out);
}

// Mat3::from_euler (vec.rs:144-149)
void oracle_mat3_from_euler(float x, float y, float z, float out_cols[9]) {
    M3<float> m = mat_mul(mat_mul(from_axis_angle(V3<float>{1, 0, 0}, x), from_axis_angle(V3<float>{0, 1, 0}, y)),
                          from_axis_angle(V3<float>{0, 0, 1}, z));
    for (int c = 0; c < 3; ++c) {
        out_cols[3 * c + 0] = m.c[c].x;
        out_cols[3 * c + 1] = m.c[c].y;
        out_cols[3 * c + 2] = m.c[c].z;
    }
}

// Quat::to_mat3 (vec.rs:318-326) after Quat::normalize (vec.rs:276-283; dot at :272-274):
// columns of the rotation matrix of the normalised quaternion (x, y, z, w).
void oracle_quat_to_mat3(const float q_xyzw[4], float out_cols[9]) {
    float x = q_xyzw[0], y = q_xyzw[1], z = q_xyzw[2], w = q_xyzw[3];
    float n = std::sqrt(x * x + y * y + z * z + w * w);
    if (n > 1e-12f) {
        x = x / n;
        y = y / n;
        z = z / n;
        w = w / n;
    } else {  // Quat::IDENTITY
        x = 0.0f;
        y = 0.0f;
        z = 0.0f;
        w = 1.0f;
    }
    const float c[9] = {1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + z * w), 2.0f * (x * z - y * w),
                        2.0f * (x * y - z * w), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + x * w),
                        2.0f * (x * z + y * w), 2.0f * (y * z - x * w), 1.0f - 2.0f * (x * x + y * y)};
    for (int i = 0; i < 9; ++i) out_cols[i] = c[i];
}

// Full frame through the reference's render() semantics: beauty (with post) or a debug AOV.
// rgba: w*h*4 floats (Framebuffer pixels). hdr3 (optional): beauty radiance before post.
int oracle_render(const mm3e_scene_desc* d, const mm3e_camera* cam, unsigned threads, float* rgba, float* hdr3) {
    Scene<float> s = scene_from_desc<float>(*d);
    if (s.materials.empty()) return -1;
    size_t n = (size_t)s.width * s.height;
    std::vector<V3<float>> hdr(hdr3 ? n : 0);
    render_frame(s, cam_from<float>(*cam), threads, rgba, hdr3 ? hdr.data() : nullptr);
    if (hdr3)
        for (size_t i = 0; i < n; ++i) {
            hdr3[3 * i] = hdr[i].x;
            hdr3[3 * i + 1] = hdr[i].y;
            hdr3[3 * i + 2] = hdr[i].z;
        }
    return 0;
}

// Beauty radiance (render_linear) for rows [y0, y1): the bounded CPU-baseline sample.
int oracle_render_rows(const mm3e_scene_desc* d, const mm3e_camera* cam, uint32_t y0, uint32_t y1, unsigned threads, float* hdr3) {
    Scene<float> s = scene_from_desc<float>(*d);
    if (s.materials.empty() || y1 < y0 || y1 > s.height) return -1;
    std::vector<V3<float>> rows((size_t)(y1 - y0) * s.width);
    render_linear_rows(s, cam_from<float>(*cam), y0, y1, threads, rows.data());
    for (size_t i = 0; i < rows.size(); ++i) {
        hdr3[3 * i] = rows[i].x;
        hdr3[3 * i + 1] = rows[i].y;
        hdr3[3 * i + 2] = rows[i].z;
    }
    return 0;
}

// post::resolve on a given HDR buffer.
int oracle_post(const mm3e_scene_desc* d, const float* hdr3, float* rgba) {
    Scene<float> s = scene_from_desc<float>(*d);
    size_t n = (size_t)s.width * s.height;
    std::vector<V3<float>> hdr(n);
    for (size_t i = 0; i < n; ++i) hdr[i] = V3<float>{hdr3[3 * i], hdr3[3 * i + 1], hdr3[3 * i + 2]};
    post_resolve(hdr, s.width, s.height, s.post, rgba);
    return 0;
}

// Primary pinhole ray through each pixel centre (the AOV / film ray): hit mask, t, matId,
// steps and normal. mat of a miss is reported as 0xFFFFFFFF.
int oracle_primary_hits(const mm3e_scene_desc* d, const mm3e_camera* cam, unsigned threads, float* t, uint32_t* mat,
                        uint32_t* steps, float* normal3) {
    Scene<float> s = scene_from_desc<float>(*d);
    Camera<float> c = cam_from<float>(*cam);
    bool dual_safe = scene_dual_safe(s);
    for_row_bands(0, s.height, threads, [&](uint32_t a, uint32_t b, size_t) {
        World<float> w(s);
        for (uint32_t y = a; y < b; ++y)
            for (uint32_t x = 0; x < s.width; ++x) {
                Ray<float> ray = camera_ray(c, (float)x + 0.5f, (float)y + 0.5f, s.width, s.height);
                Hit<float> h = march_scene(s, w, dual_safe, ray);
                size_t i = (size_t)y * s.width + x;
                t[i] = h.t;
                mat[i] = h.hit ? h.mat : 0xFFFFFFFFu;
                if (steps) steps[i] = h.steps;
                if (normal3) {
                    normal3[3 * i] = h.normal.x;
                    normal3[3 * i + 1] = h.normal.y;
                    normal3[3 * i + 2] = h.normal.z;
                }
            }
    });
    return 0;
}

// March arbitrary rays (origin xyz, dir xyz per ray) in f32 or f64 (the FP64 re-march).
int oracle_march_rays(const mm3e_scene_desc* d, const float* rays6, size_t n, int use_double, unsigned threads,
                      double* t, uint32_t* mat, uint32_t* steps, double* normal3) {
    auto run = [&](auto tag) {
        using T = decltype(tag);
        Scene<T> s = scene_from_desc<T>(*d);
        bool dual_safe = scene_dual_safe(s);
        for_row_bands(0, (uint32_t)n, threads, [&](uint32_t a, uint32_t b, size_t) {
            World<T> w(s);
            for (uint32_t i = a; i < b; ++i) {
                Ray<T> r{v3f<T>(rays6 + 6 * i), v3f<T>(rays6 + 6 * i + 3)};
                Hit<T> h = march_scene(s, w, dual_safe, r);
                t[i] = o_value(h.t);
                mat[i] = h.hit ? h.mat : 0xFFFFFFFFu;
                if (steps) steps[i] = h.steps;
                if (normal3) {
                    normal3[3 * i] = o_value(h.normal.x);
                    normal3[3 * i + 1] = o_value(h.normal.y);
                    normal3[3 * i + 2] = o_value(h.normal.z);
                }
            }
        });
    };
    if (use_double) run(double(0));
    else run(float(0));
    return 0;
}

// Soft-shadow factor, in binary32, of every (ray, light) at the ray's hit, cast as shade_hit casts
// it (lib.rs:1315-1333): lifted origin hit.pos + normal * max(2 normal_h, 0.01), toward the
// light, max_t = min(light distance, max_dist). shadow[i * n_lights + l] is -1 where no shadow ray
// is cast (a miss, a light behind the surface, shadows off); n_lights is the scene's light count.
int oracle_soft_shadows(const mm3e_scene_desc* d, const float* rays6, size_t n, unsigned threads, float* shadow) {
    Scene<float> s = scene_from_desc<float>(*d);
    bool dual_safe = scene_dual_safe(s);
    const size_t nl = s.lights.size();
    for_row_bands(0, (uint32_t)n, threads, [&](uint32_t a, uint32_t b, size_t) {
        World<float> w(s);
        for (uint32_t i = a; i < b; ++i) {
            Ray<float> r{v3f<float>(rays6 + 6 * i), v3f<float>(rays6 + 6 * i + 3)};
            Hit<float> hit = march_scene(s, w, dual_safe, r);
            for (size_t l = 0; l < nl; ++l) {
                float out = -1.0f;
                const auto& light = s.lights[l];
                V3<float> l_dir;
                float l_dist;
                if (hit.hit && s.shadows) {
                    light.toward(hit.pos, l_dir, l_dist);
                    if (lambert(hit.normal, l_dir) > 0.0f) {
                        float max_t = o_min(l_dist, s.marcher.max_dist);
                        float lift = o_max(s.marcher.normal_h * 2.0f, 0.01f);
                        out = s.marcher.soft_shadow(w, hit.pos + scale(hit.normal, lift), l_dir, max_t,
                                                    light.shadow_k(l_dist));
                    }
                }
                shadow[i * nl + l] = out;
            }
        }
    });
    return 0;
}

// Ambient occlusion, in binary32, at every ray's hit, as shade_hit takes it (lib.rs:1300-1304,
// march.rs:264-280); -1 where the ray misses or the scene has AO off.
int oracle_ambient_occlusion(const mm3e_scene_desc* d, const float* rays6, size_t n, unsigned threads, float* occ) {
    Scene<float> s = scene_from_desc<float>(*d);
    bool dual_safe = scene_dual_safe(s);
    for_row_bands(0, (uint32_t)n, threads, [&](uint32_t a, uint32_t b, size_t) {
        World<float> w(s);
        for (uint32_t i = a; i < b; ++i) {
            Ray<float> r{v3f<float>(rays6 + 6 * i), v3f<float>(rays6 + 6 * i + 3)};
            Hit<float> hit = march_scene(s, w, dual_safe, r);
            occ[i] = hit.hit && s.ao ? s.marcher.ambient_occlusion(w, hit.pos, hit.normal) : -1.0f;
        }
    });
    return 0;
}

// World field at points (accelerated WorldPlan, or the linear reference fold).
int oracle_field(const mm3e_scene_desc* d, const float* pts3, size_t n, int linear, float* dist, uint32_t* mat) {
    Scene<float> s = scene_from_desc<float>(*d);
    World<float> w(s);
    for (size_t i = 0; i < n; ++i) {
        V3<float> p = v3f<float>(pts3 + 3 * i);
        Field<float> f = linear ? w.linear(p) : w(p);
        dist[i] = f.dist;
        mat[i] = f.mat;
    }
    return 0;
}

namespace {
void put_counts(const OpCounts& t, uint64_t* out) {
    uint64_t v[14] = {t.fp32(), t.add, t.mul, t.cmp, t.minmax, t.div, t.sqrt, t.trans, t.field_evals, t.dual_evals,
                      t.primary_rays, t.reflection_rays, t.shadow_rays, t.gi_rays};
    std::memcpy(out, v, sizeof(v));
}
}  // namespace

// Operation counts for one full frame, f32 semantics, 14 values per block:
// [fp32, add, mul, cmp, minmax, div, sqrt, trans, field_evals, dual_evals,
//  primary_rays, reflection_rays, shadow_rays, gi_rays].
// Blocks: 0 render phase (tape interpretation + shading), 1 post phase (bloom + tone map),
// then the render phase split by kernel: 2 march (+ hit normal), 3 AO, 4 soft shadow of the
// primary level, 5 shading (camera rays, BRDF / IBL / GI / fog, reflection set-up, all levels),
// 6 march, 7 AO, 8 soft shadow of the reflection levels (as many blocks as `n_blocks` asks).
int oracle_count_frame_blocks(const mm3e_scene_desc* d, const mm3e_camera* cam, unsigned threads, uint64_t* counts,
                              int n_blocks) {
    Scene<CountF> s = scene_from_desc<CountF>(*d);
    Camera<CountF> c = cam_from<CountF>(*cam);
    size_t n = (size_t)s.width * s.height;
    std::vector<V3<CountF>> hdr(n);
    OpCounts render, post, phase[PH_COUNT];
    std::mutex mu;
    bool dual_safe = scene_dual_safe(s);
    for_row_bands(0, s.height, threads, [&](uint32_t a, uint32_t b, size_t) {
        reset_counts();
        World<CountF> w(s);
        for (uint32_t y = a; y < b; ++y)
            for (uint32_t x = 0; x < s.width; ++x) {
                if (s.mode == MM3E_MODE_BEAUTY) hdr[(size_t)y * s.width + x] = shade_pixel(s, w, c, x, y, dual_safe);
                else (void)aov_pixel(s, w, c, x, y, dual_safe);
            }
        std::lock_guard<std::mutex> lk(mu);
        for (int i = 0; i < PH_COUNT; ++i) {
            render.merge(phase_counts()[i]);
            phase[i].merge(phase_counts()[i]);
        }
    });
    if (s.mode == MM3E_MODE_BEAUTY) {
        reset_counts();
        std::vector<float> rgba(4 * n);
        post_resolve(hdr, s.width, s.height, s.post, rgba.data());
        for (int i = 0; i < PH_COUNT; ++i) post.merge(phase_counts()[i]);
    }
    put_counts(render, counts);
    if (n_blocks > 1) put_counts(post, counts + 14);
    for (int i = 0; i < PH_COUNT && i + 2 < n_blocks; ++i) put_counts(phase[i], counts + 14 * (i + 2));
    return 0;
}

// Render + post blocks only (28 values).
int oracle_count_frame(const mm3e_scene_desc* d, const mm3e_camera* cam, unsigned threads, uint64_t* counts) {
    return oracle_count_frame_blocks(d, cam, threads, counts, 2);
}

// Scene::bake_gi (lib.rs:665-682). cubes: nx*ny*nz*18 floats. Returns 1 if baked, 0 if the
// scene has nothing bounded (no GI), negative on error.
int oracle_bake_gi(const mm3e_scene_desc* d, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t samples, unsigned threads,
                   float* min3, float* size3, uint32_t* dims3, float* cubes) {
    Scene<float> s = scene_from_desc<float>(*d);
    GiVolume<float> g;
    if (!bake_gi(s, nx, ny, nz, samples, threads, g)) return 0;
    min3[0] = g.min.x; min3[1] = g.min.y; min3[2] = g.min.z;
    size3[0] = g.size.x; size3[1] = g.size.y; size3[2] = g.size.z;
    dims3[0] = (uint32_t)g.nx; dims3[1] = (uint32_t)g.ny; dims3[2] = (uint32_t)g.nz;
    if (cubes)
        for (size_t i = 0; i < g.cubes.size(); ++i)
            for (int f = 0; f < 6; ++f) {
                cubes[i * 18 + f * 3 + 0] = g.cubes[i][f].x;
                cubes[i * 18 + f * 3 + 1] = g.cubes[i][f].y;
                cubes[i * 18 + f * 3 + 2] = g.cubes[i][f].z;
            }
    return 1;
}

// GiVolume::sample on the scene's GI at given points/normals (known-answer tests).
int oracle_gi_sample(const mm3e_scene_desc* d, const float* pts3, const float* nrm3, size_t n, float* out3) {
    Scene<float> s = scene_from_desc<float>(*d);
    if (!s.gi) return -1;
    for (size_t i = 0; i < n; ++i) {
        V3<float> r = s.gi->sample(v3f<float>(pts3 + 3 * i), v3f<float>(nrm3 + 3 * i));
        out3[3 * i] = r.x;
        out3[3 * i + 1] = r.y;
        out3[3 * i + 2] = r.z;
    }
    return 0;
}

// ---- kit-level entry points for the reference's known-answer tests ----------------------
// sdf.rs primitive distance in local space (kind = MM3E_PRIM_* 0..10).
float oracle_sdf(uint32_t kind, const float* params, float x, float y, float z) {
    return prim_distance<float>(kind, params, V3<float>{x, y, z});
}
// sdf.rs combinators: op 0 union, 1 intersect, 2 subtract, 3 smooth_union, 4 smooth_subtract,
// 5 smooth_intersect.
void oracle_combine(uint32_t op, float ad, uint32_t am, float bd, uint32_t bm, float k, float* od, uint32_t* om) {
    Field<float> a{ad, am}, b{bd, bm}, r;
    switch (op) {
        case 0: r = f_union(a, b); break;
        case 1: r = f_intersect(a, b); break;
        case 2: r = f_subtract(a, b); break;
        case 3: r = f_smooth_union(a, b, k); break;
        case 4: {  // sdf.rs:163-170
            if (k <= 0.0f) { r = f_subtract(a, b); break; }
            float h = o_clamp(0.5f - 0.5f * (a.dist + b.dist) / k, 0.0f, 1.0f);
            r = Field<float>{a.dist * (1.0f - h) + (-b.dist) * h + k * h * (1.0f - h), a.mat};
            break;
        }
        default: {  // sdf.rs:173-181
            if (k <= 0.0f) { r = f_intersect(a, b); break; }
            float h = o_clamp(0.5f - 0.5f * (a.dist - b.dist) / k, 0.0f, 1.0f);
            r = Field<float>{a.dist * (1.0f - h) + b.dist * h + k * h * (1.0f - h), h > 0.5f ? b.mat : a.mat};
            break;
        }
    }
    *od = r.dist;
    *om = r.mat;
}
// sdf.rs domain ops: op 0 round(d=x, r=a), 1 onion(d=x, t=a), 2 elongate, 3 repeat, 4 twist,
// 5 bend, 6 mirror (a,b,c as booleans). p = xyz in/out.
void oracle_domain(uint32_t op, float* p, float a, float b, float c) {
    V3<float> v{p[0], p[1], p[2]};
    switch (op) {
        case 0: p[0] = op_round(p[0], a); return;
        case 1: p[0] = op_onion(p[0], a); return;
        case 2: v = op_elongate(v, V3<float>{a, b, c}); break;
        case 3: v = op_repeat(v, V3<float>{a, b, c}); break;
        case 4: v = op_twist(v, a); break;
        case 5: v = op_bend(v, a); break;
        default: v = op_mirror(v, a != 0.0f, b != 0.0f, c != 0.0f); break;
    }
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
// shade.rs: brdf / fresnel_schlick / aces
void oracle_brdf(const float* n, const float* l, const float* v, const float* albedo, float metallic, float roughness,
                 float reflectance, float* out3) {
    V3<float> r = brdf(v3f<float>(n), v3f<float>(l), v3f<float>(v), v3f<float>(albedo), metallic, roughness, reflectance);
    out3[0] = r.x;
    out3[1] = r.y;
    out3[2] = r.z;
}
float oracle_fresnel(float cos_theta, float f0) { return fresnel_schlick(cos_theta, f0); }
void oracle_aces(const float* in3, float* out3) {
    V3<float> r = aces(v3f<float>(in3));
    out3[0] = r.x;
    out3[1] = r.y;
    out3[2] = r.z;
}

// Wall-clock of a CPU render of rows [y0, y1) in seconds (bench CPU-baseline helper).
double oracle_time_rows(const mm3e_scene_desc* d, const mm3e_camera* cam, uint32_t y0, uint32_t y1, unsigned threads) {
    Scene<float> s = scene_from_desc<float>(*d);
    std::vector<V3<float>> rows((size_t)(y1 - y0) * s.width);
    auto t0 = std::chrono::steady_clock::now();
    render_linear_rows(s, cam_from<float>(*cam), y0, y1, threads, rows.data());
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}


// mesh.rs bake_sdf: positions (3 floats each), triangles (3 indices each). Writes the grid dims,
// min corner and cell; `data` (nx*ny*nz floats) may be NULL to query the grid only. Returns 0,
// or -1 with the reference's error message in `err`.
int oracle_bake_mesh_sdf(const float* positions, uint32_t n_positions, const uint32_t* triangles, uint32_t n_triangles,
                         uint32_t resolution, float padding, unsigned threads, uint32_t* dims, float* min3, float* cell3,
                         float* data, size_t n_floats, char* err, size_t err_len) {
    oracle::mesh::Mesh m;
    m.pos.resize(n_positions);
    for (uint32_t i = 0; i < n_positions; ++i)
        m.pos[i] = oracle::mesh::F3{positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]};
    m.tri.assign(triangles, triangles + 3 * (size_t)n_triangles);
    oracle::mesh::Grid g{};
    std::string e;
    std::vector<float> vol;
    if (data) e = oracle::mesh::bake_sdf(m, resolution, padding, g, vol, threads);
    else e = oracle::mesh::bake_grid(m, resolution, padding, g);
    if (!e.empty()) {
        if (err && err_len) {
            std::strncpy(err, e.c_str(), err_len - 1);
            err[err_len - 1] = 0;
        }
        return -1;
    }
    dims[0] = g.nx;
    dims[1] = g.ny;
    dims[2] = g.nz;
    min3[0] = g.lo.x;
    min3[1] = g.lo.y;
    min3[2] = g.lo.z;
    cell3[0] = g.cell.x;
    cell3[1] = g.cell.y;
    cell3[2] = g.cell.z;
    if (data) {
        if (n_floats < vol.size()) return -2;
        std::memcpy(data, vol.data(), vol.size() * sizeof(float));
    }
    return 0;
}

// triangle.rs x_crossing: 1 and *x when the X-directed line at (y, z) crosses the triangle.
int oracle_x_crossing(const float* a, const float* b, const float* c, float y, float z, float* x) {
    return oracle::mesh::x_crossing(oracle::mesh::F3{a[0], a[1], a[2]}, oracle::mesh::F3{b[0], b[1], b[2]},
                                    oracle::mesh::F3{c[0], c[1], c[2]}, y, z, *x)
               ? 1
               : 0;
}


// film.rs render_film: beauty3 / foreground3 / normals3 (3 floats per pixel), alpha, depth (+inf
// on a miss), mat_ids (0xFFFFFFFF on a miss); any output may be NULL. Returns 0, or -1 with an
// invalid lens (Lens::validate).
int oracle_render_film(const mm3e_scene_desc* d, const mm3e_camera* cam, float aperture_radius, float focus_distance,
                       unsigned threads, float* beauty3, float* fg3, float* alpha, float* depth, float* normals3,
                       uint32_t* mat_ids) {
    if (!std::isfinite(aperture_radius) || aperture_radius < 0.0f) return -1;
    if (!std::isfinite(focus_distance) || focus_distance <= 0.0f) return -1;
    Scene<float> s = scene_from_desc<float>(*d);
    Camera<float> c = cam_from<float>(*cam);
    bool dual_safe = scene_dual_safe(s);
    for_row_bands(0, s.height, threads, [&](uint32_t a, uint32_t b, size_t) {
        World<float> w(s);
        for (uint32_t y = a; y < b; ++y)
            for (uint32_t x = 0; x < s.width; ++x) {
                FilmSample<float> f = film_sample_pixel(s, w, c, aperture_radius, focus_distance, x, y, dual_safe);
                size_t i = (size_t)y * s.width + x;
                if (beauty3) std::memcpy(beauty3 + 3 * i, &f.beauty, 12);
                if (fg3) std::memcpy(fg3 + 3 * i, &f.foreground, 12);
                if (alpha) alpha[i] = f.alpha;
                if (depth) depth[i] = f.center.hit ? dot(f.center.pos - c.eye, c.forward) : INFINITY;
                if (normals3) {
                    V3<float> nrm = f.center.hit ? f.center.normal : zero3<float>();
                    std::memcpy(normals3 + 3 * i, &nrm, 12);
                }
                if (mat_ids) mat_ids[i] = f.center.hit ? f.center.mat : 0xFFFFFFFFu;
            }
    });
    return 0;
}


namespace {
// render_gbuffer's per-pixel display value (lib.rs:1016-1018)
inline void display_u8(V3<float> hdr, float exposure, uint8_t* px) {
    V3<float> d = clamp01(gamma(aces(scale(hdr, exposure))));
    px[0] = (uint8_t)(d.x * 255.0f + 0.5f);
    px[1] = (uint8_t)(d.y * 255.0f + 0.5f);
    px[2] = (uint8_t)(d.z * 255.0f + 0.5f);
    px[3] = 255;
}

// reproject.rs:55-70
inline bool project(const Camera<float>& c, V3<float> world, uint32_t w, uint32_t h, float& sx, float& sy, float& fz) {
    V3<float> v = world - c.eye;
    fz = dot(v, c.forward);
    if (fz <= 1e-4f) return false;
    float aspect = (float)w / (float)h;
    float ndc_x = dot(v, c.right) / fz;
    float ndc_y = dot(v, c.up) / fz;
    sx = (ndc_x / (aspect * c.fov_scale) + 1.0f) * 0.5f * (float)w;
    sy = (1.0f - ndc_y / c.fov_scale) * 0.5f * (float)h;
    return true;
}
}  // namespace

// render_gbuffer (lib.rs:951-1039): display RGBA8, primary hit distance (+inf: sky), mover
// index (-1: none) per pixel; movers4 = (centre xyz, radius) per mover.
int oracle_render_gbuffer(const mm3e_scene_desc* d, const mm3e_camera* cam, const float* movers4, uint32_t n_movers,
                          unsigned threads, uint8_t* color4, float* depth, int32_t* obj) {
    Scene<float> s = scene_from_desc<float>(*d);
    Camera<float> c = cam_from<float>(*cam);
    bool dual_safe = scene_dual_safe(s);
    for_row_bands(0, s.height, threads, [&](uint32_t a, uint32_t b, size_t) {
        World<float> w(s);
        for (uint32_t y = a; y < b; ++y)
            for (uint32_t x = 0; x < s.width; ++x) {
                size_t i = (size_t)y * s.width + x;
                Ray<float> ray = camera_ray(c, (float)x + 0.5f, (float)y + 0.5f, s.width, s.height);
                Hit<float> hit = march_scene(s, w, dual_safe, ray, 0);
                V3<float> hdr;
                if (hit.hit) {
                    int32_t o = -1;
                    for (uint32_t k = 0; k < n_movers; ++k) {
                        V3<float> ctr{movers4[4 * k], movers4[4 * k + 1], movers4[4 * k + 2]};
                        if (length(hit.pos - ctr) <= movers4[4 * k + 3] + 0.05f) {
                            o = (int32_t)k;
                            break;
                        }
                    }
                    hdr = shade_hit(s, w, hit, ray, 0, dual_safe);
                    depth[i] = hit.t;
                    obj[i] = o;
                } else {
                    hdr = sky(ray.dir, s.sun_dir);
                    depth[i] = INFINITY;
                    obj[i] = -1;
                }
                display_u8(hdr, s.post.exposure, color4 + 4 * i);
            }
    });
    return 0;
}

// reproject::warp (reproject.rs:77-113): out color4 and filled (0/1) per pixel of the new view.
int oracle_reproject_warp(uint32_t w, uint32_t h, const mm3e_camera* prev_cam, const uint8_t* color4,
                          const float* depth, const int32_t* obj, const mm3e_camera* new_cam, const float* deltas3,
                          uint32_t n_deltas, uint8_t* out4, uint8_t* filled) {
    Camera<float> pc = cam_from<float>(*prev_cam), nc = cam_from<float>(*new_cam);
    size_t n = (size_t)w * h;
    std::vector<float> zbuf(n, INFINITY);
    std::memset(out4, 0, 4 * n);
    std::memset(filled, 0, n);
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            size_t i = (size_t)y * w + x;
            V3<float> dir = camera_ray(pc, (float)x + 0.5f, (float)y + 0.5f, w, h).dir;
            float dd = std::isfinite(depth[i]) ? depth[i] : 1.0e6f;
            V3<float> world = pc.eye + scale(dir, dd);
            if (obj[i] >= 0 && (uint32_t)obj[i] < n_deltas)
                world = world + V3<float>{deltas3[3 * obj[i]], deltas3[3 * obj[i] + 1], deltas3[3 * obj[i] + 2]};
            float sx, sy, fz;
            if (!project(nc, world, w, h, sx, sy, fz)) continue;
            int32_t nx = (int32_t)std::floor(sx), ny = (int32_t)std::floor(sy);
            if (nx >= 0 && ny >= 0 && (uint32_t)nx < w && (uint32_t)ny < h) {
                size_t j = (size_t)ny * w + nx;
                if (fz < zbuf[j]) {
                    zbuf[j] = fz;
                    std::memcpy(out4 + 4 * j, color4 + 4 * i, 4);
                    filled[j] = 1;
                }
            }
        }
    return 0;
}

// reproject::reproject's row hole fill (reproject.rs:118-146), in place.
int oracle_reproject_fill(uint32_t w, uint32_t h, uint8_t* out4, uint8_t* filled) {
    for (uint32_t y = 0; y < h; ++y) {
        bool have = false;
        uint8_t last[4];
        for (uint32_t x = 0; x < w; ++x) {
            size_t i = (size_t)y * w + x;
            if (filled[i]) {
                std::memcpy(last, out4 + 4 * i, 4);
                have = true;
            } else if (have) {
                std::memcpy(out4 + 4 * i, last, 4);
                filled[i] = 1;
            }
        }
        have = false;
        for (uint32_t x = w; x-- > 0;) {
            size_t i = (size_t)y * w + x;
            if (filled[i]) {
                std::memcpy(last, out4 + 4 * i, 4);
                have = true;
            } else if (have) {
                std::memcpy(out4 + 4 * i, last, 4);
            }
        }
    }
    return 0;
}

// reproject_hybrid's hole rerender (lib.rs:1047-1080): every unfilled pixel is marched and
// shaded at the new camera, in place.
int oracle_rerender_holes(const mm3e_scene_desc* d, const mm3e_camera* new_cam, unsigned threads, uint8_t* out4,
                          const uint8_t* filled) {
    Scene<float> s = scene_from_desc<float>(*d);
    Camera<float> c = cam_from<float>(*new_cam);
    bool dual_safe = scene_dual_safe(s);
    for_row_bands(0, s.height, threads, [&](uint32_t a, uint32_t b, size_t) {
        World<float> w(s);
        for (uint32_t y = a; y < b; ++y)
            for (uint32_t x = 0; x < s.width; ++x) {
                size_t i = (size_t)y * s.width + x;
                if (filled[i]) continue;
                Ray<float> ray = camera_ray(c, (float)x + 0.5f, (float)y + 0.5f, s.width, s.height);
                Hit<float> hit = march_scene(s, w, dual_safe, ray, 0);
                V3<float> hdr = hit.hit ? shade_hit(s, w, hit, ray, 0, dual_safe) : sky(ray.dir, s.sun_dir);
                display_u8(hdr, s.post.exposure, out4 + 4 * i);
            }
    });
    return 0;
}

}  // extern "C"
