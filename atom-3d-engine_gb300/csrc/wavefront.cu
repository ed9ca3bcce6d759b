// wavefront.cu — sm_103a wavefront kernels of the MM3E per-pixel SDF render path.
//
// A frame is a short sequence of small kernels over ray queues. Keeping each kernel's code
// footprint small matters more here than anything else: a single kernel holding the march,
// the shadow march, AO and all of the shading stalls on instruction fetch.
//
// The march and shadow kernels are persistent tape interpreters: each CTA stages the scene
// tape into shared memory with TMA bulk copies (cp.async.bulk) completing on an mbarrier, and
// every lane runs one ray at a time, one field sample per loop iteration; a lane that
// finishes refills from a global counter with one warp-aggregated atomic (ballot + popc +
// shfl), so warps stay full without a separate compaction pass.
#include <cuda_runtime.h>

#include "../../include/mm3e_cuda.h"
#include "device_math.cuh"
#include "kernels.h"

namespace mm3e {
namespace {

constexpr int WAVE_THREADS = 128;
constexpr uint32_t SMEM_TAPE_MAX = 96 * 1024;

__device__ __forceinline__ uint32_t item_count(const WaveArgs& a) { return a.n_items_dev ? *a.n_items_dev : a.n_items; }

// Bounded wait on an mbarrier phase; false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Stage the tape into shared memory: TMA bulk copies (<= 32 KB each) completing on one
// mbarrier, waited on with an iteration limit. Returns false (status word set) on failure.
__device__ __forceinline__ bool stage_tape(unsigned char* smem, const unsigned char* tape, uint32_t bytes,
                                           uint32_t* status) {
    __shared__ __align__(8) uint64_t mbar_storage;
    __shared__ uint32_t tape_ok;
    uint32_t mbar = (uint32_t)__cvta_generic_to_shared(&mbar_storage);
    uint32_t dst = (uint32_t)__cvta_generic_to_shared(smem);
    if (threadIdx.x == 0) {
        tape_ok = 1u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
        for (uint32_t off = 0; off < bytes; off += 32768u) {
            uint32_t n = bytes - off < 32768u ? bytes - off : 32768u;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    dst + off),
                "l"(tape + off), "r"(n), "r"(mbar)
                : "memory");
        }
    }
    if (!mbar_wait(mbar, 0u, 1u << 22)) tape_ok = 0u;
    __syncthreads();
    bool ok = tape_ok && reinterpret_cast<const TapeHeader*>(smem)->magic == TAPE_MAGIC;
    if (!ok && threadIdx.x == 0) atomicOr(status, tape_ok ? ST_TAPE_CORRUPT : ST_TAPE_TIMEOUT);
    return ok;
}

// Warp-aggregated refill of idle lanes: returns false once the lane is retired.
__device__ __forceinline__ void refill(uint32_t& item, bool& retired, uint32_t n, uint32_t* counter, bool& fresh) {
    fresh = false;
    const uint32_t lane = threadIdx.x & 31u;
    unsigned want = __ballot_sync(0xFFFFFFFFu, item == NIL && !retired);
    if (!want) return;
    uint32_t base = 0;
    int leader = __ffs(want) - 1;
    if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(want));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (item == NIL && !retired) {
        uint32_t it = base + (uint32_t)__popc(want & ((1u << lane) - 1u));
        if (it >= n) retired = true;
        else {
            item = it;
            fresh = true;
        }
    }
}

// Camera::ray (camera.rs:59-65)
__device__ __forceinline__ V camera_dir(const CameraArgs& c, float sx, float sy, uint32_t w, uint32_t h) {
    float wf = (float)w, hf = (float)h;
    float aspect = wf / hf;
    float ndc_x = (2.0f * sx / wf - 1.0f) * aspect * c.fov_scale;
    float ndc_y = (1.0f - 2.0f * sy / hf) * c.fov_scale;
    return normalize(ld3(c.fwd) + scale(ld3(c.right), ndc_x) + scale(ld3(c.up), ndc_y));
}

// Pixel of a tiled pixel index (8x4 tiles, row-major tiles); false for padding pixels.
__device__ __forceinline__ bool tiled_pixel(uint32_t p, uint32_t w, uint32_t h, uint32_t& x, uint32_t& y) {
    uint32_t tiles_x = (w + 7u) / 8u;
    uint32_t tile = p >> 5, r = p & 31u;
    x = (tile % tiles_x) * 8u + (r & 7u);
    y = (tile / tiles_x) * 4u + (r >> 3);
    return x < w && y < h;
}

__device__ __forceinline__ V tetra_k(uint32_t t) {
    // k0 = (1,-1,-1), k1 = (-1,-1,1), k2 = (-1,1,-1), k3 = (1,1,1) (march.rs:212-223)
    return V{(t == 0u || t == 3u) ? 1.0f : -1.0f, (t >= 2u) ? 1.0f : -1.0f, (t == 1u || t == 3u) ? 1.0f : -1.0f};
}

// ------------------------------------------------------------------------------------------
// march: enhanced sphere tracing (march.rs:120-209) + hit normal (march.rs:212-223 or
// Scene::normal_dual, lib.rs:820-835), one ray per lane.
// ------------------------------------------------------------------------------------------
constexpr uint32_t M_IDLE = 0, M_MARCH = 1, M_COVER = 2, M_TETRA = 3;
constexpr uint32_t BOOST_OMEGA = 0, BOOST_LEAP = 1, BOOST_SECANT = 2;

struct MLane {
    uint32_t item, phase;
    V ro, rd;
    float t, prev_r, step, t_prev, d_prev, omega, subz;
    uint32_t i, secant_on, boost;
    float sv_d, sv_r, sv_e;
    uint32_t sv_m, hmat;
    V g;
    uint32_t tap;
};

__device__ __forceinline__ V m_at(const MLane& L, float t) { return L.ro + scale(L.rd, t); }

// Finish a ray: write the hit record (normal, t, material or NIL, steps).
__device__ __forceinline__ void m_write(MLane& L, const WaveArgs& a, bool hit, V n, uint32_t steps) {
    a.b.h_n[L.item] = make_float4(n.x, n.y, n.z, L.t);
    a.b.h_m[L.item] = make_uint2(hit ? L.hmat : NIL, steps);
    L.item = NIL;
    L.phase = M_IDLE;
}

template <bool SMEM>
__global__ void __launch_bounds__(WAVE_THREADS) k_march(const __grid_constant__ WaveArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned char* tape = a.tape;
    if (SMEM) {
        if (!stage_tape(smem, a.tape, a.tape_bytes, a.status)) return;
        tape = smem;
    }
    const Tape T = tape_view(tape);
    const TapeHeader& h = *T.h;
    const uint32_t n = item_count(a);
    const uint32_t max_steps = h.max_steps;
    MLane L;
    L.item = NIL;
    L.phase = M_IDLE;
    bool retired = false;
    for (;;) {
        bool fresh;
        refill(L.item, retired, n, a.counter, fresh);
        if (__ballot_sync(0xFFFFFFFFu, !retired) == 0u) break;
        if (fresh) {
            // ray for the item
            if (a.src == SRC_SAMPLES) {
                uint32_t aa = h.aa, spp = aa * aa;
                uint32_t pix = L.item / spp, sub = L.item % spp;
                uint32_t x, y;
                bool inside = tiled_pixel(pix, h.width, h.height, x, y);
                uint32_t sx = sub % aa, sy = sub / aa;
                float nf = (float)aa;
                float ox = ((float)sx + 0.5f) / nf, oy = ((float)sy + 0.5f) / nf;
                L.ro = ld3(a.cam.eye);
                L.rd = inside ? camera_dir(a.cam, (float)x + ox, (float)y + oy, h.width, h.height) : V{0.f, 0.f, 1.f};
                a.b.q_o[L.item] = make_float4(L.ro.x, L.ro.y, L.ro.z, __uint_as_float(L.item));
                a.b.q_d[L.item] = make_float4(L.rd.x, L.rd.y, L.rd.z, 0.0f);
                if (!inside) {  // padding pixel of the last tile row / column
                    L.t = 0.0f;
                    m_write(L, a, false, V{0.f, 0.f, 0.f}, 0u);
                    continue;
                }
            } else if (a.src == SRC_CENTER) {
                uint32_t x = L.item % h.width, y = L.item / h.width;
                L.ro = ld3(a.cam.eye);
                L.rd = camera_dir(a.cam, (float)x + 0.5f, (float)y + 0.5f, h.width, h.height);
                a.b.q_o[L.item] = make_float4(L.ro.x, L.ro.y, L.ro.z, __uint_as_float(L.item));
                a.b.q_d[L.item] = make_float4(L.rd.x, L.rd.y, L.rd.z, 0.0f);
            } else if (a.src == SRC_QUEUE) {
                float4 o = a.b.q_o[L.item], d = a.b.q_d[L.item];
                L.ro = V{o.x, o.y, o.z};
                L.rd = V{d.x, d.y, d.z};
            } else {  // SRC_GATHER (gi.rs:75-87)
                uint32_t dpf = a.dirs_per_face;
                uint32_t dd = L.item % dpf, rest = L.item / dpf;
                uint32_t face = rest % 6u, probe = rest / 6u;
                uint32_t i = probe % a.gi_nx, j = (probe / a.gi_nx) % a.gi_ny, k = probe / (a.gi_nx * a.gi_ny);
                L.ro = ld3(a.gi_lo) + V{(float)i * a.gi_cell[0], (float)j * a.gi_cell[1], (float)k * a.gi_cell[2]};
                float4 dw = a.gather_dirs[face * dpf + dd];
                L.rd = V{dw.x, dw.y, dw.z};
                a.b.q_o[L.item] = make_float4(L.ro.x, L.ro.y, L.ro.z, __uint_as_float(L.item));
                a.b.q_d[L.item] = make_float4(L.rd.x, L.rd.y, L.rd.z, 0.0f);
            }
            // march.rs:132-141
            L.t = 0.0f;
            L.prev_r = 0.0f;
            L.step = 0.0f;
            L.t_prev = 0.0f;
            L.d_prev = __int_as_float(0x7f800000);
            bool lip = h.step_scale >= 1.0f;
            L.omega = lip ? 1.4f : h.step_scale;
            L.subz = lip ? h.subitize : 0.0f;
            L.secant_on = ((h.flags & SF_SECANT) && lip) ? 1u : 0u;
            L.boost = BOOST_OMEGA;
            L.i = 0;
            L.phase = M_MARCH;
            if (max_steps == 0) m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
        }
        if (L.phase == M_IDLE) continue;
        V p;
        if (L.phase == M_MARCH) p = m_at(L, L.t);
        else if (L.phase == M_COVER) p = m_at(L, 0.5f * ((L.t_prev + L.prev_r) + (L.t - L.sv_r)));
        else p = m_at(L, L.t) + scale(tetra_k(L.tap), h.normal_h);
        Field f = world_eval(T, p);
        // ---- advance ----
        if (L.phase == M_TETRA) {
            V kd = scale(tetra_k(L.tap), f.d);
            L.g = L.tap == 0 ? kd : L.g + kd;
            L.tap += 1;
            if (L.tap == 4u) m_write(L, a, true, normalize(L.g), L.i);
            continue;
        }
        float d;
        uint32_t m;
        float radius, e;
        if (L.phase == M_MARCH) {
            d = f.d;
            m = f.m;
            radius = fabsf(d);
            e = h.eps * (1.0f + L.t * 0.5f) + h.lod_footprint * L.t;
            bool overlap_fail = (L.step > 0.0f && d < 0.0f) || L.step > radius + L.prev_r;
            if (overlap_fail && d > 0.0f) {  // check the gap midpoint first
                L.sv_d = d;
                L.sv_m = m;
                L.sv_r = radius;
                L.sv_e = e;
                L.phase = M_COVER;
                continue;
            }
            if (overlap_fail) goto rollback;
        } else {  // M_COVER
            float gap_lo = L.t_prev + L.prev_r;
            float gap_hi = L.t - L.sv_r;
            L.phase = M_MARCH;
            if (!(f.d >= 0.5f * (gap_hi - gap_lo))) goto rollback;
            d = L.sv_d;
            m = L.sv_m;
            radius = L.sv_r;
            e = L.sv_e;
        }
        // march.rs:173-206
        if (d < e) {
            L.hmat = m;
            if (h.flags & SF_DUAL_SAFE) {
                m_write(L, a, true, normal_dual(T.obj, h.n_objects, m_at(L, L.t)), L.i);
            } else {
                L.phase = M_TETRA;
                L.tap = 0;
            }
            continue;
        }
        {
            float step_len = d * L.omega;
            uint32_t boost = BOOST_OMEGA;
            if (L.subz > 0.0f && d > e * 6.0f) {
                step_len = step_len * (1.0f + L.subz);
                boost = BOOST_LEAP;
            }
            if (L.secant_on && d < 0.08f && isfinite(L.d_prev)) {
                float dt = L.t - L.t_prev;
                float dd = d - L.d_prev;
                if (dt > 1e-6f && dd < -1e-6f) {
                    step_len = clampf(-d * dt / dd, d, d * 4.0f);
                    boost = BOOST_SECANT;
                }
            }
            L.step = step_len;
            L.boost = boost;
            L.prev_r = radius;
            L.d_prev = d;
            L.t_prev = L.t;
            L.t = L.t + step_len;
            if (L.t > h.max_dist) {
                m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
                continue;
            }
            L.i += 1;
            if (L.i >= max_steps) m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
            continue;
        }
    rollback:  // retreat to the last safe frontier (march.rs:155-170)
        L.t = L.t_prev + L.prev_r;
        if (L.boost == BOOST_OMEGA) L.omega = fminf(L.omega, 1.0f);
        else if (L.boost == BOOST_LEAP) L.subz = 0.0f;
        else L.secant_on = 0;
        L.boost = BOOST_OMEGA;
        L.prev_r = 0.0f;
        L.step = 0.0f;
        L.d_prev = __int_as_float(0x7f800000);
        L.i += 1;
        if (L.i >= max_steps) m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
    }
}

// ------------------------------------------------------------------------------------------
// ao: Marcher::ambient_occlusion (march.rs:264-280) at every hit
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(WAVE_THREADS) k_ao(const __grid_constant__ WaveArgs a) {
    const Tape T = tape_view(a.tape);
    const TapeHeader& h = *T.h;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= item_count(a)) return;
    uint2 hm = a.b.h_m[slot];
    if (hm.x == NIL) {
        a.b.occ[slot] = 1.0f;
        return;
    }
    float4 hn4 = a.b.h_n[slot], o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
    V hp = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
    V n{hn4.x, hn4.y, hn4.z};
    uint32_t ns = h.ao_samples;
    float base = fmaxf(h.normal_h, 0.01f);
    float span = (float)((ns > 2u ? ns : 2u) - 1u);
    float occ = 0.0f, sca = 1.0f;
    for (uint32_t i = 0; i < ns; ++i) {
        float hr = base + 0.12f * (float)i / span;
        float d = world_eval(T, hp + scale(n, hr)).d;
        occ = occ + (hr - d) * sca;
        sca = sca * 0.92f;
    }
    a.b.occ[slot] = ns == 0 ? 1.0f : clampf(1.0f - 2.6f * occ, 0.0f, 1.0f);
}

// ------------------------------------------------------------------------------------------
// shadow: Marcher::soft_shadow (march.rs:227-259) per (hit, light), one march per lane
// ------------------------------------------------------------------------------------------
template <bool SMEM>
__global__ void __launch_bounds__(WAVE_THREADS) k_shadow(const __grid_constant__ WaveArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const unsigned char* tape = a.tape;
    if (SMEM) {
        if (!stage_tape(smem, a.tape, a.tape_bytes, a.status)) return;
        tape = smem;
    }
    const Tape T = tape_view(tape);
    const TapeHeader& h = *T.h;
    const uint32_t nl = h.n_lights;
    const uint32_t n = item_count(a) * nl;
    uint32_t item = NIL;
    bool retired = false;
    V so, sdir;
    float st = 0.f, sres = 1.f, sk = 0.f, smax = 0.f;
    uint32_t si = 0;
    for (;;) {
        bool fresh;
        refill(item, retired, n, a.counter, fresh);
        if (__ballot_sync(0xFFFFFFFFu, !retired) == 0u) break;
        if (fresh) {
            uint32_t slot = item / nl, li = item % nl;
            uint2 hm = a.b.h_m[slot];
            bool live = false;
            if (hm.x != NIL) {
                float4 hn4 = a.b.h_n[slot], o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
                V hp = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
                V hn{hn4.x, hn4.y, hn4.z};
                const DevLight& lt = T.light[li];
                V ldir;
                float ldist;
                light_toward(lt, hp, ldir, ldist);
                if (fmaxf(dot(hn, ldir), 0.0f) > 0.0f) {  // lib.rs:1315-1322
                    float lift = fmaxf(h.normal_h * 2.0f, 0.01f);
                    so = hp + scale(hn, lift);
                    sdir = ldir;
                    smax = fminf(ldist, h.max_dist);
                    sk = light_shadow_k(lt, ldist);
                    float hb = so.x * 127.1f + so.y * 311.7f + so.z * 74.7f;
                    float sv = sinf(hb) * 43758.547f;
                    st = 0.02f + fabsf(sv - truncf(sv)) * 0.16f;
                    sres = 1.0f;
                    si = 0;
                    live = true;
                }
            }
            if (!live) {
                a.b.shadow[item] = -1.0f;
                item = NIL;
                continue;
            }
        }
        if (item == NIL) continue;
        float hh = world_eval(T, so + scale(sdir, st)).d;
        if (hh < 0.0008f) {
            a.b.shadow[item] = 0.0f;
            item = NIL;
            continue;
        }
        sres = fminf(sres, sk * hh / st);
        st = st + clampf(hh, 0.06f, 0.5f + 0.7f * st);
        si += 1;
        if (st > smax || si >= h.shadow_steps) {
            a.b.shadow[item] = clampf(sres, 0.0f, 1.0f);
            item = NIL;
        }
    }
}

// ------------------------------------------------------------------------------------------
// shade: shade_hit (lib.rs:1286-1360) / sky on a miss; reflection rays go to the next queue
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(WAVE_THREADS) k_shade(const __grid_constant__ WaveArgs a) {
    const Tape T = tape_view(a.tape);
    const TapeHeader& h = *T.h;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    bool active = slot < item_count(a);
    bool emit = false;
    V rorig{0.f, 0.f, 0.f}, rdir{0.f, 0.f, 0.f};
    uint32_t sample = 0;
    if (active) {
        float4 o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
        sample = __float_as_uint(o4.w);
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
                float shadow = shadows ? a.b.shadow[(size_t)slot * h.n_lights + li] : 1.0f;
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
                size_t li = ((size_t)level * a.n_samples + sample) * 2;
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
            a.b.nq_d[q] = make_float4(rdir.x, rdir.y, rdir.z, 0.0f);
        }
    }
}

// ------------------------------------------------------------------------------------------
// resolve: fold reflection levels (lib.rs:1353-1359) and average AA samples (lib.rs:1231-1242)
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(WAVE_THREADS) k_resolve(const __grid_constant__ WaveArgs a, uint32_t w, uint32_t hh) {
    const TapeHeader* h = reinterpret_cast<const TapeHeader*>(a.tape);
    uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t x, y;
    uint32_t tiles = ((w + 7u) / 8u) * ((hh + 3u) / 4u) * 32u;
    if (pix >= tiles || !tiled_pixel(pix, w, hh, x, y)) return;
    uint32_t aa = h->aa, spp = aa * aa;
    V fog = ld3(h->fog);
    float density = h->fog_density;
    V acc{0.f, 0.f, 0.f};
    for (uint32_t sub = 0; sub < spp; ++sub) {
        uint32_t s = pix * spp + sub;
        float4 t4 = a.b.term[s];
        V v{t4.x, t4.y, t4.z};
        uint32_t lvl = __float_as_uint(t4.w);
        while (lvl > 0) {
            lvl -= 1;
            size_t li = ((size_t)lvl * a.n_samples + s) * 2;
            float4 A = a.b.lvl[li], B = a.b.lvl[li + 1];
            V r = scale(V{A.x, A.y, A.z}, 1.0f - A.w) + scale(v, A.w);
            r = r + V{B.x, B.y, B.z};
            v = apply_fog(r, fog, B.w, density);
        }
        acc = acc + v;
    }
    V o = scale(acc, 1.0f / (float)spp);
    a.b.hdr[(size_t)y * w + x] = make_float4(o.x, o.y, o.z, 1.0f);
}

// AOV display values (lib.rs:1185-1217) for pixel-centre hits (row-major slots).
__global__ void __launch_bounds__(WAVE_THREADS) k_aov(const __grid_constant__ WaveArgs a, uint32_t w, uint32_t hh,
                                                      float4* out) {
    const Tape T = tape_view(a.tape);
    const TapeHeader& h = *T.h;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= w * hh) return;
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
__global__ void __launch_bounds__(WAVE_THREADS) k_gather_shade(const __grid_constant__ WaveArgs a, float4* radiance) {
    const Tape T = tape_view(a.tape);
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
// Post (post.rs:36-115)
// ---------------------------------------------------------------------------------------
__global__ void k_bright(const float4* __restrict__ hdr, float4* __restrict__ bright, size_t n, float thr) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 c = hdr[i];
    V v{c.x, c.y, c.z};
    float l = luminance(v);
    V b{0.f, 0.f, 0.f};
    if (l > thr) b = scale(v, (l - thr) / fmaxf(l, 1e-4f));
    bright[i] = make_float4(b.x, b.y, b.z, 0.0f);
}

// One separable pass with clamped borders (post.rs:348-368); taps summed in kernel order.
template <bool HORIZONTAL>
__global__ void k_blur(const float4* __restrict__ src, float4* __restrict__ dst, const float* __restrict__ kw,
                       uint32_t radius, uint32_t w, uint32_t h) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    int r = (int)radius;
    V acc{0.f, 0.f, 0.f};
    for (int ki = 0; ki <= 2 * r; ++ki) {
        int off = ki - r;
        int sx = HORIZONTAL ? min(max((int)x + off, 0), (int)w - 1) : (int)x;
        int sy = HORIZONTAL ? (int)y : min(max((int)y + off, 0), (int)h - 1);
        float4 s = __ldg(src + (size_t)sy * w + sx);
        acc = acc + scale(V{s.x, s.y, s.z}, __ldg(kw + ki));
    }
    dst[(size_t)y * w + x] = make_float4(acc.x, acc.y, acc.z, 0.0f);
}

__device__ __forceinline__ unsigned char to_u8(float c) {
    return (unsigned char)__float2uint_rz(clampf(c, 0.0f, 1.0f) * 255.0f + 0.5f);
}

__global__ void k_resolve_post(const float4* __restrict__ hdr, const float4* __restrict__ bloom, size_t n,
                               float intensity, float exposure, int format, void* out) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 c = hdr[i];
    V col{c.x, c.y, c.z};
    if (bloom) {
        float4 b = bloom[i];
        col = col + scale(V{b.x, b.y, b.z}, intensity);
    }
    V d = display(col, exposure);
    if (format == MM3E_FB_RGBA8) reinterpret_cast<uchar4*>(out)[i] = make_uchar4(to_u8(d.x), to_u8(d.y), to_u8(d.z), 255);
    else reinterpret_cast<float4*>(out)[i] = make_float4(d.x, d.y, d.z, 1.0f);
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

template <class K>
cudaError_t launch_persistent(K kernel_smem, K kernel_global, const WaveArgs& a, cudaStream_t s, int sm_count) {
    bool use_smem = a.tape_bytes <= SMEM_TAPE_MAX;
    size_t smem = use_smem ? a.tape_bytes : 0;
    if (use_smem && smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TAPE_MAX);
        if (e != cudaSuccess) return e;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, use_smem ? kernel_smem : kernel_global,
                                                                  WAVE_THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint32_t blocks = (uint32_t)(per_sm * sm_count);
    if (!a.n_items_dev) {
        uint32_t needed = (a.n_items + WAVE_THREADS - 1) / WAVE_THREADS;
        if (needed < blocks) blocks = needed > 0 ? needed : 1;
    }
    if (use_smem) kernel_smem<<<blocks, WAVE_THREADS, smem, s>>>(a);
    else kernel_global<<<blocks, WAVE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

unsigned grid_for(uint32_t n) { return (n + WAVE_THREADS - 1) / WAVE_THREADS > 0 ? (n + WAVE_THREADS - 1) / WAVE_THREADS : 1; }

}  // namespace

cudaError_t launch_march(const WaveArgs& a, cudaStream_t s, int sm_count, uint32_t* launches) {
    if (launches) *launches += 1;
    return launch_persistent(k_march<true>, k_march<false>, a, s, sm_count);
}

cudaError_t launch_shadow(const WaveArgs& a, cudaStream_t s, int sm_count, uint32_t* launches) {
    if (launches) *launches += 1;
    return launch_persistent(k_shadow<true>, k_shadow<false>, a, s, sm_count);
}

// Non-persistent kernels are sized for the largest queue (a.n_items) and read the live count
// from n_items_dev when set.
cudaError_t launch_ao(const WaveArgs& a, cudaStream_t s, uint32_t* launches) {
    if (launches) *launches += 1;
    k_ao<<<grid_for(a.n_items), WAVE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_shade(const WaveArgs& a, cudaStream_t s, uint32_t* launches) {
    if (launches) *launches += 1;
    k_shade<<<grid_for(a.n_items), WAVE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const WaveArgs& a, uint32_t width, uint32_t height, cudaStream_t s, uint32_t* launches) {
    uint32_t tiles = ((width + 7u) / 8u) * ((height + 3u) / 4u) * 32u;
    if (launches) *launches += 1;
    k_resolve<<<grid_for(tiles), WAVE_THREADS, 0, s>>>(a, width, height);
    return cudaGetLastError();
}

cudaError_t launch_aov(const WaveArgs& a, uint32_t width, uint32_t height, float4* out, cudaStream_t s,
                       uint32_t* launches) {
    if (launches) *launches += 1;
    k_aov<<<grid_for(width * height), WAVE_THREADS, 0, s>>>(a, width, height, out);
    return cudaGetLastError();
}

cudaError_t launch_gather_shade(const WaveArgs& a, float4* radiance, cudaStream_t s, uint32_t* launches) {
    if (launches) *launches += 1;
    k_gather_shade<<<grid_for(a.n_items), WAVE_THREADS, 0, s>>>(a, radiance);
    return cudaGetLastError();
}

cudaError_t launch_post(const PostArgs& p, cudaStream_t s, uint32_t* launches) {
    size_t n = (size_t)p.width * p.height;
    if (n == 0) return cudaSuccess;
    unsigned blocks = (unsigned)((n + 255) / 256);
    const float4* bloom = nullptr;
    if (p.bloom) {
        k_bright<<<blocks, 256, 0, s>>>(p.hdr, p.bright, n, p.threshold);
        dim3 b2(32, 8), g2((p.width + 31) / 32, (p.height + 7) / 8);
        k_blur<true><<<g2, b2, 0, s>>>(p.bright, p.blur_h, p.kernel_w, p.radius, p.width, p.height);
        k_blur<false><<<g2, b2, 0, s>>>(p.blur_h, p.bright, p.kernel_w, p.radius, p.width, p.height);
        bloom = p.bright;
        if (launches) *launches += 3;
    }
    k_resolve_post<<<blocks, 256, 0, s>>>(p.hdr, bloom, n, p.intensity, p.exposure, p.format, p.out);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_pack_rgba8(const float4* src, uchar4* dst, size_t n, cudaStream_t s, uint32_t* launches) {
    if (n == 0) return cudaSuccess;
    k_pack8<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, n);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_field(const unsigned char* tape, uint32_t tape_bytes, const float* pts, uint32_t n, float* dist,
                         uint32_t* mat, cudaStream_t s, uint32_t* launches) {
    (void)tape_bytes;
    if (n == 0) return cudaSuccess;
    k_field<<<(n + 127) / 128, 128, 0, s>>>(tape, pts, n, dist, mat);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_gi_reduce(const float4* radiance, const float4* dirs, uint32_t dirs_per_face, uint32_t probes,
                             float4* cubes, cudaStream_t s, uint32_t* launches) {
    uint32_t n = probes * 6u;
    if (n == 0) return cudaSuccess;
    k_gi_reduce<<<(n + 127) / 128, 128, 0, s>>>(radiance, dirs, dirs_per_face, probes, cubes);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

}  // namespace mm3e
