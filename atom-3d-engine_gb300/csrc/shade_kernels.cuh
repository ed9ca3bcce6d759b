// shade_kernels.cuh — per-slot bodies of the shading, reflection-emit and resolve passes of the
// wavefront render path (shade_hit, lib.rs:1286-1360; trace, lib.rs:1265-1282; the AA average,
// lib.rs:1223-1243), of the AOV display modes, and of the GI bake's gather shading and per-face
// average. The kernels that run them over a pass's slots are in wavefront.cu; the bodies take
// their arguments and one slot, so a host loop can drive them slot by slot as well.
#pragma once
#include "../../include/mm3e_cuda.h"
#include "march_kernels.cuh"

namespace mm3e {
namespace wave {

// ------------------------------------------------------------------------------------------
// shade: shade_hit (lib.rs:1286-1360) / sky on a miss; reflection rays go to the next queue
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void shade_slots(const WaveArgs& a, uint32_t slot, bool active) {
    bool emit = false;
    V rorig{0.f, 0.f, 0.f}, rdir{0.f, 0.f, 0.f};
    uint32_t sample = 0, job = 0;
    if (active) {
        float4 o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
        sample = __float_as_uint(o4.w);
        job = a.jobs ? __float_as_uint(d4.w) : 0u;
        const Tape T = tape_view(job_ref(a, job).tape);
        const TapeHeader& h = *T.h;
        V rd{d4.x, d4.y, d4.z};
        uint2 hm = a.b.h_m[slot];
        uint32_t level = a.level;
        if (hm.x == NIL) {
            V v = sky(rd, ld3(h.sun_dir));
            a.b.term[sample] = make_float4(v.x, v.y, v.z, __uint_as_float(level));
        } else {
            float4 hn4 = a.b.h_n[slot];
            float ht = hn4.w;
            V hp = V{o4.x, o4.y, o4.z} + scale(rd, ht);
            V hn{hn4.x, hn4.y, hn4.z};
            const DevMaterial& m = T.mat[hm.x % h.n_materials];
            V albedo = surface_albedo(m, hp);
            V view = scale(rd, -1.0f);
            // The AO pass runs where the scene has AO and AO samples; without samples
            // ambient_occlusion is 1 (march.rs:266), as without AO.
            float occ = ((h.flags & SF_AO) && h.ao_samples > 0u) ? a.b.occ[slot] : 1.0f;
            V gi = V{0.f, 0.f, 0.f};
            if (h.flags & SF_GI) gi = gi_sample(h, hp, hn);
            V amb = ibl_irradiance(hn, ld3(h.sun_dir), ld3(h.sky_ambient)) + gi + ld3(h.ambient);
            V rad = scale(cmul(albedo, amb), occ);
            bool shadows = (h.flags & SF_SHADOWS) && h.shadow_steps > 0;
            for (uint32_t li = 0; li < h.n_lights; ++li) {
                const DevLight& lt = T.light[li];
                V ldir;
                float ldist;
                light_toward(lt, hp, ldir, ldist);
                if (fmaxf(dot(hn, ldir), 0.0f) <= 0.0f) continue;
                float shadow = shadows ? a.b.shadow[(size_t)slot * a.lights_max + li] : 1.0f;
                if (shadow <= 0.0f) continue;
                V surface = brdf(hn, ldir, view, albedo, m.metallic, m.roughness, m.specular);
                rad = rad + scale(cmul(surface, ld3(lt.color)), shadow * light_atten(lt, ldist));
            }
            V em = ld3(m.emissive);
            if (level < h.bounces && m.reflectivity > 0.0f) {
                float cosv = fmaxf(dot(hn, view), 0.0f);
                float fr = fresnel_schlick(cosv, m.reflectivity);
                rdir = normalize(reflect(rd, hn));
                rorig = hp + scale(hn, fmaxf(h.normal_h * 2.0f, 0.02f));
                size_t li = ((size_t)level * a.cap + sample) * 2;
                a.b.lvl[li] = make_float4(rad.x, rad.y, rad.z, fr);
                a.b.lvl[li + 1] = make_float4(em.x, em.y, em.z, ht);
                emit = true;
            } else {
                V v = apply_fog(rad + em, ld3(h.fog), ht, h.fog_density);
                a.b.term[sample] = make_float4(v.x, v.y, v.z, __uint_as_float(level));
            }
        }
    }
    // append reflection rays to the next level's queue (one atomic per warp)
    if (!a.emit) return;
    const uint32_t lane = threadIdx.x & 31u;
    unsigned mask = __ballot_sync(0xFFFFFFFFu, emit);
    if (mask) {
        uint32_t base = 0;
        int leader = __ffs(mask) - 1;
        if ((int)lane == leader) base = atomicAdd(a.b.nq_count, (uint32_t)__popc(mask));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (emit) {
            uint32_t q = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
            a.b.nq_o[q] = make_float4(rorig.x, rorig.y, rorig.z, __uint_as_float(sample));
            a.b.nq_d[q] = make_float4(rdir.x, rdir.y, rdir.z, __uint_as_float(job));
        }
    }
}

// The reflection ray shade_hit recurses into (lib.rs:1336-1343), emitted as soon as the level's
// hits exist so the next level can march while this level's AO / shadows / shading run.
__device__ __forceinline__ void reflect_slots(const WaveArgs& a, uint32_t slot, bool active) {
    bool emit = false;
    V rorig{0.f, 0.f, 0.f}, rdir{0.f, 0.f, 0.f};
    uint32_t sample = 0, job = 0;
    if (active) {
        uint2 hm = a.b.h_m[slot];
        if (hm.x != NIL) {
            float4 o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
            job = a.jobs ? __float_as_uint(d4.w) : 0u;
            const Tape T = tape_view(job_ref(a, job).tape);
            const TapeHeader& h = *T.h;
            const DevMaterial& m = T.mat[hm.x % h.n_materials];
            if (a.level < h.bounces && m.reflectivity > 0.0f) {
                sample = __float_as_uint(o4.w);
                float4 hn4 = a.b.h_n[slot];
                V rd{d4.x, d4.y, d4.z};
                V hp = V{o4.x, o4.y, o4.z} + scale(rd, hn4.w);
                V hn{hn4.x, hn4.y, hn4.z};
                rdir = normalize(reflect(rd, hn));
                rorig = hp + scale(hn, fmaxf(h.normal_h * 2.0f, 0.02f));
                emit = true;
            }
        }
    }
    const uint32_t lane = threadIdx.x & 31u;
    unsigned mask = __ballot_sync(0xFFFFFFFFu, emit);
    if (mask) {
        uint32_t base = 0;
        int leader = __ffs(mask) - 1;
        if ((int)lane == leader) base = atomicAdd(a.b.nq_count, (uint32_t)__popc(mask));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (emit) {
            uint32_t q = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
            a.b.nq_o[q] = make_float4(rorig.x, rorig.y, rorig.z, __uint_as_float(sample));
            a.b.nq_d[q] = make_float4(rdir.x, rdir.y, rdir.z, __uint_as_float(job));
        }
    }
}

// ------------------------------------------------------------------------------------------
// resolve: fold reflection levels (lib.rs:1353-1359) and average AA samples (lib.rs:1231-1242)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void resolve_slot(const WaveArgs& a, uint32_t slot, uint32_t nj) {
    const FrameJob& J = job_ref(a, a.jobs ? find_job<1>(a.jobs, nj, slot) : 0u);
    uint32_t p = slot - J.slot_base;
    uint32_t x, y;
    if (!tiled_pixel(p, J, a.tile_wlog, x, y)) return;
    const TapeHeader* h = reinterpret_cast<const TapeHeader*>(J.tape);  // fog
    uint32_t spp = J.spp;
    V fog = ld3(h->fog);
    float density = h->fog_density;
    V acc{0.f, 0.f, 0.f}, fg{0.f, 0.f, 0.f};
    uint32_t hits = 0;
    for (uint32_t sub = 0; sub < spp; ++sub) {
        uint32_t s = J.sample_base + p * spp + sub;
        float4 t4 = a.b.term[s];
        V v{t4.x, t4.y, t4.z};
        uint32_t lvl = __float_as_uint(t4.w);
        while (lvl > 0) {
            lvl -= 1;
            size_t li = ((size_t)lvl * a.cap + s) * 2;
            float4 A = a.b.lvl[li], B = a.b.lvl[li + 1];
            V r = scale(V{A.x, A.y, A.z}, 1.0f - A.w) + scale(v, A.w);
            r = r + V{B.x, B.y, B.z};
            v = apply_fog(r, fog, B.w, density);
        }
        acc = acc + v;
        if (a.film && a.b.h_m[s].x != NIL) {  // film.rs:182-190: coverage of primary hits
            fg = fg + v;
            hits += 1;
        }
    }
    float inv = 1.0f / (float)spp;
    V o = scale(acc, inv);
    size_t px = (size_t)J.pixel_base + (size_t)y * J.width + x;
    if (a.film) {
        V f = scale(fg, inv);
        a.b.hdr[px] = make_float4(o.x, o.y, o.z, (float)hits * inv);
        a.b.fg[px] = make_float4(f.x, f.y, f.z, 0.0f);
    } else {
        a.b.hdr[px] = make_float4(o.x, o.y, o.z, 1.0f);
    }
}

// ------------------------------------------------------------------------------------------
// GI bake: Scene::gather (lib.rs:686-711) at a gather ray's hit, and the per-face average
// (GiVolume::bake, gi.rs:78-86)
// ------------------------------------------------------------------------------------------
// Emissive plus unshadowed direct light at the hit, or the diffuse sky on a miss.
__device__ __forceinline__ void gather_slot(const WaveArgs& a, uint32_t slot, float4* radiance) {
    const Tape T = tape_view(a.job0.tape);
    const TapeHeader& h = *T.h;
    float4 o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
    V rd{d4.x, d4.y, d4.z};
    uint2 hm = a.b.h_m[slot];
    V c;
    if (hm.x == NIL) {
        c = sky_diffuse(rd, ld3(h.sun_dir));
    } else {
        float4 hn4 = a.b.h_n[slot];
        V hp = V{o4.x, o4.y, o4.z} + scale(rd, hn4.w);
        V hn{hn4.x, hn4.y, hn4.z};
        const DevMaterial& m = T.mat[hm.x % h.n_materials];
        V albedo = surface_albedo(m, hp);
        c = ld3(m.emissive);
        V view = scale(rd, -1.0f);
        for (uint32_t li = 0; li < h.n_lights; ++li) {
            const DevLight& lt = T.light[li];
            V ldir;
            float ldist;
            light_toward(lt, hp, ldir, ldist);
            if (fmaxf(dot(hn, ldir), 0.0f) > 0.0f) {
                V out = brdf(hn, ldir, view, albedo, m.metallic, m.roughness, m.specular);
                c = c + scale(cmul(out, ld3(lt.color)), light_atten(lt, ldist));
            }
        }
    }
    radiance[slot] = make_float4(c.x, c.y, c.z, 0.0f);
}

// Weighted average of one probe face's gather radiances (idx = probe * 6 + face), summed in
// direction order.
__device__ __forceinline__ void gi_reduce_slot(const float4* __restrict__ rad, const float4* __restrict__ dirs,
                                               uint32_t dpf, uint32_t idx, float4* __restrict__ cubes) {
    uint32_t face = idx % 6u;
    V acc{0.f, 0.f, 0.f};
    float wsum = 0.0f;
    for (uint32_t d = 0; d < dpf; ++d) {
        float4 r = rad[(size_t)idx * dpf + d];
        float w = dirs[face * dpf + d].w;
        acc = acc + scale(V{r.x, r.y, r.z}, w);
        wsum = wsum + w;
    }
    V c = scale(acc, 1.0f / fmaxf(wsum, 1e-4f));
    cubes[idx] = make_float4(c.x, c.y, c.z, 0.0f);
}

// ------------------------------------------------------------------------------------------
// AOV display value (lib.rs:1185-1217) of a pixel-centre hit of job 0 (row-major slots)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void aov_slot(const WaveArgs& a, uint32_t slot, float4* out) {
    const Tape T = tape_view(a.job0.tape);
    const TapeHeader& h = *T.h;
    uint2 hm = a.b.h_m[slot];
    float4 hn4 = a.b.h_n[slot];
    bool hit = hm.x != NIL;
    V n{hn4.x, hn4.y, hn4.z};
    V v{0.f, 0.f, 0.f};
    switch (a.aov_mode) {
        case MM3E_MODE_NORMAL: v = hit ? scale(n, 0.5f) + splat(0.5f) : V{0.f, 0.f, 0.f}; break;
        case MM3E_MODE_DEPTH: v = splat(1.0f - clampf(hn4.w / h.max_dist, 0.0f, 1.0f)); break;
        case MM3E_MODE_AO: v = hit ? splat(a.b.occ[slot]) : splat(1.0f); break;
        case MM3E_MODE_STEPS: {
            float t = clampf((float)hm.y / (float)h.max_steps, 0.0f, 1.0f);
            v = V{clampf(t * 3.0f - 1.5f, 0.f, 1.f), clampf(1.0f - fabsf(t * 3.0f - 1.3f), 0.f, 1.f),
                  clampf(1.0f - t * 2.2f, 0.f, 1.f)};
            break;
        }
        default: {
            if (hit) {
                float4 o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
                V hp = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
                v = surface_albedo(T.mat[hm.x % h.n_materials], hp);
            }
            break;
        }
    }
    v = clamp01(v);
    out[slot] = make_float4(v.x, v.y, v.z, 1.0f);
}

}  // namespace wave
}  // namespace mm3e
