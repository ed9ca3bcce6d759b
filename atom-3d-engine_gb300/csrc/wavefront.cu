// wavefront.cu — sm_103a wavefront kernels of the MM3E per-pixel SDF render path.
//
// A frame is a short sequence of small kernels over ray queues. Keeping each kernel's code
// footprint small matters more here than anything else: a single kernel holding the march,
// the shadow march, AO and all of the shading stalls on instruction fetch. The march,
// shadow and AO bodies live in march_kernels.cuh (shared with the scene-specialised NVRTC
// program); this file instantiates them with the tape interpreter and holds the shading,
// resolve, AOV, GI and post kernels.
#include <cuda_runtime.h>

#include "../../include/mm3e_cuda.h"
#include "kernels.h"
#include "march_kernels.cuh"

namespace mm3e {
namespace {

using namespace wave;

template <int TM, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) k_march(const __grid_constant__ WaveArgs a) {
    march_body<TM, UNROLL, InterpField>(a);
}

template <int TM, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) k_shadow(const __grid_constant__ WaveArgs a) {
    shadow_body<TM, UNROLL, InterpField>(a);
}

__global__ void __launch_bounds__(SHADE_THREADS) k_ao(const __grid_constant__ WaveArgs a) { ao_body<InterpField>(a); }

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
            float occ = (h.flags & SF_AO) ? a.b.occ[slot] : 1.0f;
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

__global__ void __launch_bounds__(SHADE_THREADS) k_shade(const __grid_constant__ WaveArgs a) {
    const uint32_t n = item_count(a);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
        shade_slots(a, base + threadIdx.x, base + threadIdx.x < n);  // block-uniform trip count
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

__global__ void __launch_bounds__(SHADE_THREADS) k_reflect(const __grid_constant__ WaveArgs a) {
    const uint32_t n = item_count(a);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
        reflect_slots(a, base + threadIdx.x, base + threadIdx.x < n);
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

__global__ void __launch_bounds__(SHADE_THREADS) k_resolve(const __grid_constant__ WaveArgs a, uint32_t n_slots) {
    uint32_t nj = 1;
    if (a.jobs) {
        n_slots = a.totals->n_slots;
        nj = a.totals->n_jobs;
    }
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n_slots; slot += gridDim.x * blockDim.x)
        resolve_slot(a, slot, nj);
}

// AOV display values (lib.rs:1185-1217) for pixel-centre hits of job 0 (row-major slots).
__global__ void __launch_bounds__(SHADE_THREADS) k_aov(const __grid_constant__ WaveArgs a, float4* out) {
    const Tape T = tape_view(a.job0.tape);
    const TapeHeader& h = *T.h;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= a.job0.width * a.job0.height) return;
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

// Scene::gather (lib.rs:686-711): emissive + unshadowed direct light, or the diffuse sky.
__global__ void __launch_bounds__(SHADE_THREADS) k_gather_shade(const __grid_constant__ WaveArgs a, float4* radiance) {
    const Tape T = tape_view(a.job0.tape);
    const TapeHeader& h = *T.h;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= a.n_items) return;
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

// ---------------------------------------------------------------------------------------
// Post (post.rs:36-115), over the output pixels of every job of the pass sequence
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t post_pixels(const PostArgs& p) { return p.jobs ? p.totals->n_pixels : p.n_pixels; }
__device__ __forceinline__ const FrameJob* post_job(const PostArgs& p, uint32_t i) {
    return p.jobs ? &p.jobs[find_job<2>(p.jobs, p.totals->n_jobs, i)] : &p.job0;
}
#define MM3E_POST_LOOP(i, p)                                              \
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, n_ = post_pixels(p); i < n_; \
         i += gridDim.x * blockDim.x)

__global__ void __launch_bounds__(POST_THREADS) k_bright(const __grid_constant__ PostArgs p) {
    MM3E_POST_LOOP(i, p) {
        const FrameJob* J = post_job(p, i);
        if (!(J->flags & JF_BLOOM)) continue;
        float4 c = p.hdr[i];
        V v{c.x, c.y, c.z};
        float l = luminance(v);
        float thr = J->threshold;
        V b{0.f, 0.f, 0.f};
        if (l > thr) b = scale(v, (l - thr) / fmaxf(l, 1e-4f));
        p.bright[i] = make_float4(b.x, b.y, b.z, 0.0f);
    }
}

// One separable pass with clamped borders (post.rs:348-368); taps summed in kernel order.
template <bool HORIZONTAL>
__global__ void __launch_bounds__(POST_THREADS) k_blur(const __grid_constant__ PostArgs p, const float4* __restrict__ src,
                                                       float4* __restrict__ dst) {
    MM3E_POST_LOOP(i, p) {
        const FrameJob* J = post_job(p, i);
        if (!(J->flags & JF_BLOOM)) continue;
        uint32_t w = J->width, h = J->height;
        uint32_t local = i - J->pixel_base;
        int x = (int)(local % w), y = (int)(local / w);
        const float4* img = src + J->pixel_base;
        const float* kw = J->bloom_w;
        int r = (int)J->bloom_radius;
        V acc{0.f, 0.f, 0.f};
        for (int ki = 0; ki <= 2 * r; ++ki) {
            int off = ki - r;
            int sx = HORIZONTAL ? min(max(x + off, 0), (int)w - 1) : x;
            int sy = HORIZONTAL ? y : min(max(y + off, 0), (int)h - 1);
            float4 s = __ldg(img + (size_t)sy * w + sx);
            acc = acc + scale(V{s.x, s.y, s.z}, __ldg(kw + ki));
        }
        dst[i] = make_float4(acc.x, acc.y, acc.z, 0.0f);
    }
}

__device__ __forceinline__ unsigned char to_u8(float c) {
    return (unsigned char)__float2uint_rz(clampf(c, 0.0f, 1.0f) * 255.0f + 0.5f);
}

__global__ void __launch_bounds__(POST_THREADS) k_resolve_post(const __grid_constant__ PostArgs p) {
    MM3E_POST_LOOP(i, p) {
        const FrameJob* J = post_job(p, i);
        if (!J->out) continue;
        float4 c = p.hdr[i];
        V col{c.x, c.y, c.z};
        if (J->flags & JF_BLOOM) {
            float4 b = p.bright[i];
            col = col + scale(V{b.x, b.y, b.z}, J->intensity);
        }
        V d = display(col, J->exposure);
        uint32_t local = i - J->pixel_base;
        if (J->format == MM3E_FB_RGBA8)
            reinterpret_cast<uchar4*>(J->out)[local] = make_uchar4(to_u8(d.x), to_u8(d.y), to_u8(d.z), 255);
        else reinterpret_cast<float4*>(J->out)[local] = make_float4(d.x, d.y, d.z, 1.0f);
    }
}

__global__ void k_pack8(const float4* __restrict__ src, uchar4* __restrict__ dst, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 c = src[i];
    dst[i] = make_uchar4(to_u8(c.x), to_u8(c.y), to_u8(c.z), 255);
}

__global__ void k_field(const unsigned char* __restrict__ tape, const float* __restrict__ pts, uint32_t n,
                        float* __restrict__ dist, uint32_t* __restrict__ mat) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Tape T = tape_view(tape);
    Field f = world_eval(T, V{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    dist[i] = f.d;
    mat[i] = f.m;
}

// GiVolume::bake per-face average (gi.rs:78-86).
__global__ void k_gi_reduce(const float4* __restrict__ rad, const float4* __restrict__ dirs, uint32_t dpf,
                            uint32_t probes, float4* __restrict__ cubes) {
    uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;  // probe*6 + face
    if (idx >= probes * 6u) return;
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

typedef void (*WaveKernel)(const WaveArgs);

// Instantiations of a persistent kernel over (tape mode, block, unroll).
// Samples a lane steps between refills: the tuning's unroll rounded down to 1, 16 or 64. Long
// runs keep the warp in the step loop, whose field code then stays in the instruction cache
// (measured: 32 to 64 samples per refill cut the specialised frame times by 30-45%).
constexpr int unroll_index(uint32_t u) { return u >= 64 ? 2 : (u >= 16 ? 1 : 0); }

struct PersistentSet {
    WaveKernel k[2][2][3];  // [tape mode][block 128 / 256][unroll 1 / 16 / 64]
};

#define MM3E_PERSISTENT_SET(K)                                                                             \
    PersistentSet {                                                                                        \
        {{{K<TM_SMEM, 128, 1>, K<TM_SMEM, 128, 16>, K<TM_SMEM, 128, 64>},                                  \
          {K<TM_SMEM, 256, 1>, K<TM_SMEM, 256, 16>, K<TM_SMEM, 256, 64>}},                                 \
         {{K<TM_MULTI, 128, 1>, K<TM_MULTI, 128, 16>, K<TM_MULTI, 128, 64>},                               \
          {K<TM_MULTI, 256, 1>, K<TM_MULTI, 256, 16>, K<TM_MULTI, 256, 64>}}}                              \
    }

// Grid of a persistent launch: every CTA the SMs hold at once, fewer when the host knows
// that fewer items exist.
cudaError_t persistent_grid(const void* k, int block, size_t smem, const WaveArgs& a, int sm_count,
                            uint32_t items_per_item, uint32_t* blocks_out) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint32_t blocks = (uint32_t)(per_sm * sm_count);
    if (!a.n_items_dev) {
        uint64_t items = (uint64_t)a.n_items * items_per_item;
        uint64_t needed = (items + block - 1) / block;
        if (needed < blocks) blocks = needed > 0 ? (uint32_t)needed : 1u;
    }
    *blocks_out = blocks;
    return cudaSuccess;
}

cudaError_t launch_persistent(const PersistentSet& set, const WaveArgs& a, const TuneParams& t, cudaStream_t s,
                              int sm_count, uint32_t items_per_item) {
    bool use_smem = !a.jobs && a.tape_bytes <= SMEM_TAPE_MAX;
    int bi = t.block >= 256 ? 1 : 0;
    int ui = unroll_index(t.unroll);
    int block = bi ? 256 : 128;
    WaveKernel k = set.k[use_smem ? 0 : 1][bi][ui];
    size_t smem = use_smem ? a.tape_bytes : 0;
    if (use_smem && smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TAPE_MAX);
        if (e != cudaSuccess) return e;
    }
    uint32_t blocks = 0;
    cudaError_t e = persistent_grid(reinterpret_cast<const void*>(k), block, smem, a, sm_count, items_per_item, &blocks);
    if (e != cudaSuccess) return e;
    k<<<blocks, block, smem, s>>>(a);
    return cudaGetLastError();
}

// A specialised (run-time compiled) persistent kernel.
cudaError_t launch_persistent_spec(const void* k, const SpecKernels& sp, const WaveArgs& a, cudaStream_t s,
                                   int sm_count, uint32_t items_per_item) {
    size_t smem = sp.smem_tape ? a.tape_bytes : 0;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TAPE_MAX);
        if (e != cudaSuccess) return e;
    }
    uint32_t blocks = 0;
    cudaError_t e = persistent_grid(k, (int)sp.block, smem, a, sm_count, items_per_item, &blocks);
    if (e != cudaSuccess) return e;
    WaveArgs arg = a;
    void* args[] = {&arg};
    return cudaLaunchKernel(k, dim3(blocks), dim3(sp.block), args, smem, s);
}

unsigned grid_for(uint64_t n, int threads, uint32_t cap = 0) {
    uint64_t g = (n + threads - 1) / threads;
    if (cap && g > cap) g = cap;
    return g > 0 ? (unsigned)g : 1u;
}

}  // namespace

cudaError_t launch_march(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log,
                         const SpecKernels* spec) {
    static const PersistentSet set = MM3E_PERSISTENT_SET(k_march);
    LogScope sc(log, a.level == 0 ? KK_MARCH : KK_MARCH_REFL, s, 1);
    if (spec && spec->march && !a.jobs) return launch_persistent_spec(spec->march, *spec, a, s, sm_count, 1);
    return launch_persistent(set, a, t, s, sm_count, 1);
}

cudaError_t launch_shadow(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log,
                          const SpecKernels* spec) {
    static const PersistentSet set = MM3E_PERSISTENT_SET(k_shadow);
    LogScope sc(log, a.level == 0 ? KK_SHADOW : KK_SHADOW_REFL, s, 1);
    uint32_t per = a.lights_max ? a.lights_max : 1;
    if (spec && spec->shadow && !a.jobs) return launch_persistent_spec(spec->shadow, *spec, a, s, sm_count, per);
    return launch_persistent(set, a, t, s, sm_count, per);
}

// Non-persistent kernels are sized for the largest queue (a.n_items) and read the live count
// from n_items_dev when set.
cudaError_t launch_ao(const WaveArgs& a, cudaStream_t s, LaunchLog* log, const SpecKernels* spec) {
    LogScope sc(log, a.level == 0 ? KK_AO : KK_AO_REFL, s, 1);
    unsigned grid = grid_for(a.n_items, SHADE_THREADS, a.grid_cap);
    if (spec && spec->ao && !a.jobs) {
        WaveArgs arg = a;
        void* args[] = {&arg};
        return cudaLaunchKernel(spec->ao, dim3(grid), dim3(SHADE_THREADS), args, 0, s);
    }
    k_ao<<<grid, SHADE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_shade(const WaveArgs& a, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_SHADE, s, 1);
    k_shade<<<grid_for(a.n_items, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_reflect(const WaveArgs& a, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_SHADE, s, 1);
    k_reflect<<<grid_for(a.n_items, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const WaveArgs& a, uint32_t n_slots, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_RESOLVE, s, 1);
    k_resolve<<<grid_for(n_slots, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a, n_slots);
    return cudaGetLastError();
}

cudaError_t launch_aov(const WaveArgs& a, float4* out, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_AOV, s, 1);
    k_aov<<<grid_for((uint64_t)a.job0.width * a.job0.height, SHADE_THREADS), SHADE_THREADS, 0, s>>>(a, out);
    return cudaGetLastError();
}

cudaError_t launch_gather_shade(const WaveArgs& a, float4* radiance, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_GI, s, 1);
    k_gather_shade<<<grid_for(a.n_items, SHADE_THREADS), SHADE_THREADS, 0, s>>>(a, radiance);
    return cudaGetLastError();
}

cudaError_t launch_post(const PostArgs& p, cudaStream_t s, LaunchLog* log) {
    if (p.n_pixels == 0) return cudaSuccess;
    LogScope sc(log, KK_POST, s, p.any_bloom ? 4u : 1u);
    unsigned blocks = grid_for(p.n_pixels, POST_THREADS, p.grid_cap);
    if (p.any_bloom) {
        k_bright<<<blocks, POST_THREADS, 0, s>>>(p);
        k_blur<true><<<blocks, POST_THREADS, 0, s>>>(p, p.bright, p.blur_h);
        k_blur<false><<<blocks, POST_THREADS, 0, s>>>(p, p.blur_h, p.bright);
    }
    k_resolve_post<<<blocks, POST_THREADS, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_pack_rgba8(const float4* src, uchar4* dst, size_t n, cudaStream_t s, LaunchLog* log) {
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 1);
    k_pack8<<<grid_for(n, POST_THREADS), POST_THREADS, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_field(const unsigned char* tape, const float* pts, uint32_t n, float* dist, uint32_t* mat,
                         cudaStream_t s, LaunchLog* log) {
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 1);
    k_field<<<grid_for(n, 128), 128, 0, s>>>(tape, pts, n, dist, mat);
    return cudaGetLastError();
}

cudaError_t launch_gi_reduce(const float4* radiance, const float4* dirs, uint32_t dirs_per_face, uint32_t probes,
                             float4* cubes, cudaStream_t s, LaunchLog* log) {
    uint32_t n = probes * 6u;
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_GI, s, 1);
    k_gi_reduce<<<grid_for(n, 128), 128, 0, s>>>(radiance, dirs, dirs_per_face, probes, cubes);
    return cudaGetLastError();
}

}  // namespace mm3e
