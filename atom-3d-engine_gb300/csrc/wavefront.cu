// wavefront.cu — sm_103a wavefront kernels of the MM3E per-pixel SDF render path.
//
// A frame is a short sequence of small kernels over ray queues. Keeping each kernel's code
// footprint small matters more here than anything else: a single kernel holding the march,
// the shadow march, AO and all of the shading stalls on instruction fetch.
//
// The march and shadow kernels are persistent tape interpreters: every lane runs one ray at a
// time, one field sample per loop iteration (or `unroll` samples between refills); a lane that
// finishes refills from a global counter with one warp-aggregated atomic (ballot + popc +
// shfl), so warps stay full without a separate compaction pass. With a single job whose tape
// fits, each CTA first stages the tape into shared memory with TMA bulk copies
// (cp.async.bulk) completing on an mbarrier; with many jobs (batched / served pass sequences)
// every lane carries its ray's job and reads that job's tape through the L1 cache.
#include <cuda_runtime.h>

#include "../../include/mm3e_cuda.h"
#include "device_math.cuh"
#include "kernels.h"

namespace mm3e {
namespace {

constexpr uint32_t SMEM_TAPE_MAX = 96 * 1024;
constexpr int SHADE_THREADS = 128;
constexpr int POST_THREADS = 256;

// Tape access modes of the persistent kernels.
enum : int { TM_SMEM = 0, TM_MULTI = 1 };

__device__ __forceinline__ uint32_t item_count(const WaveArgs& a) { return a.n_items_dev ? *a.n_items_dev : a.n_items; }

__device__ __forceinline__ const FrameJob& job_ref(const WaveArgs& a, uint32_t j) { return a.jobs ? a.jobs[j] : a.job0; }

// Job holding position `x` of a job-table range (0: samples, 1: pixel slots, 2: pixels).
template <int FIELD> __device__ __forceinline__ uint32_t find_job(const FrameJob* jobs, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1u) >> 1;
        uint32_t base = FIELD == 0 ? jobs[mid].sample_base : FIELD == 1 ? jobs[mid].slot_base : jobs[mid].pixel_base;
        if (base <= x) lo = mid;
        else hi = mid - 1u;
    }
    return lo;
}

// Job of a queue slot (its index is carried in the ray direction's w).
__device__ __forceinline__ uint32_t slot_job(const WaveArgs& a, uint32_t slot) {
    return a.jobs ? __float_as_uint(a.b.q_d[slot].w) : 0u;
}

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

// Warp-aggregated refill of idle lanes; a lane retires once the items run out.
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

// Pixel of a job's pixel slot (tiles of 32 pixels, 2^wlog wide, row-major tiles); false for
// padding slots.
__device__ __forceinline__ bool tiled_pixel(uint32_t p, const FrameJob& J, uint32_t wlog, uint32_t& x, uint32_t& y) {
    uint32_t tile = p >> 5, r = p & 31u;
    uint32_t tw = 1u << wlog;
    x = (tile % J.tiles_x) * tw + (r & (tw - 1u));
    y = (tile / J.tiles_x) * (32u >> wlog) + (r >> wlog);
    return x < J.width && y < J.height;
}

__device__ __forceinline__ V tetra_k(uint32_t t) {
    // k0 = (1,-1,-1), k1 = (-1,-1,1), k2 = (-1,1,-1), k3 = (1,1,1) (march.rs:212-223)
    return V{(t == 0u || t == 3u) ? 1.0f : -1.0f, (t >= 2u) ? 1.0f : -1.0f, (t == 1u || t == 3u) ? 1.0f : -1.0f};
}

// Tape of a lane: one staged tape for the CTA (TM_SMEM) or the lane's job's tape (TM_MULTI).
template <int TM> struct LaneTape;
template <> struct LaneTape<TM_SMEM> {
    Tape T;
    __device__ __forceinline__ const Tape& get() const { return T; }
    __device__ __forceinline__ void set(const unsigned char*) {}
};
template <> struct LaneTape<TM_MULTI> {
    const unsigned char* p;
    __device__ __forceinline__ Tape get() const { return tape_view(p); }
    __device__ __forceinline__ void set(const unsigned char* tp) { p = tp; }
};

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

// Start the lane's ray for its fresh item; false when the item needs no march.
template <int TM>
__device__ __forceinline__ bool m_start(MLane& L, LaneTape<TM>& LT, const WaveArgs& a) {
    uint32_t job = 0;
    if (a.src == SRC_SAMPLES) {
        job = a.jobs ? find_job<0>(a.jobs, a.totals->n_jobs, L.item) : 0u;
        const FrameJob& J = job_ref(a, job);
        uint32_t local = L.item - J.sample_base;
        uint32_t aa = J.aa, spp = J.spp;
        uint32_t pix = local / spp, sub = local % spp;
        uint32_t x, y;
        bool inside = tiled_pixel(pix, J, a.tile_wlog, x, y);
        uint32_t sx = sub % aa, sy = sub / aa;
        float nf = (float)aa;
        float ox = ((float)sx + 0.5f) / nf, oy = ((float)sy + 0.5f) / nf;
        L.ro = ld3(J.cam.eye);
        L.rd = inside ? camera_dir(J.cam, (float)x + ox, (float)y + oy, J.width, J.height) : V{0.f, 0.f, 1.f};
        a.b.q_o[L.item] = make_float4(L.ro.x, L.ro.y, L.ro.z, __uint_as_float(L.item));
        a.b.q_d[L.item] = make_float4(L.rd.x, L.rd.y, L.rd.z, __uint_as_float(job));
        if (!inside) {  // padding pixel of the last tile row / column
            L.t = 0.0f;
            m_write(L, a, false, V{0.f, 0.f, 0.f}, 0u);
            return false;
        }
        LT.set(J.tape);
    } else if (a.src == SRC_CENTER) {
        const FrameJob& J = a.job0;
        uint32_t x = L.item % J.width, y = L.item / J.width;
        L.ro = ld3(J.cam.eye);
        L.rd = camera_dir(J.cam, (float)x + 0.5f, (float)y + 0.5f, J.width, J.height);
        a.b.q_o[L.item] = make_float4(L.ro.x, L.ro.y, L.ro.z, __uint_as_float(L.item));
        a.b.q_d[L.item] = make_float4(L.rd.x, L.rd.y, L.rd.z, 0.0f);
        LT.set(J.tape);
    } else if (a.src == SRC_QUEUE) {
        float4 o = a.b.q_o[L.item], d = a.b.q_d[L.item];
        L.ro = V{o.x, o.y, o.z};
        L.rd = V{d.x, d.y, d.z};
        job = a.jobs ? __float_as_uint(d.w) : 0u;
        LT.set(job_ref(a, job).tape);
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
        LT.set(a.job0.tape);
    }
    const TapeHeader& h = *LT.get().h;
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
    if (h.max_steps == 0) {
        m_write(L, a, false, V{0.f, 0.f, 0.f}, 0u);
        return false;
    }
    return true;
}

// One field sample of the lane's ray and the state transition it causes.
template <int TM>
__device__ __forceinline__ void m_step(MLane& L, const LaneTape<TM>& LT, const WaveArgs& a) {
    const Tape T = LT.get();
    const TapeHeader& h = *T.h;
    const uint32_t max_steps = h.max_steps;
    V p;
    if (L.phase == M_MARCH) p = m_at(L, L.t);
    else if (L.phase == M_COVER) p = m_at(L, 0.5f * ((L.t_prev + L.prev_r) + (L.t - L.sv_r)));
    else p = m_at(L, L.t) + scale(tetra_k(L.tap), h.normal_h);
    Field f = world_eval(T, p);
    if (L.phase == M_TETRA) {
        V kd = scale(tetra_k(L.tap), f.d);
        L.g = L.tap == 0 ? kd : L.g + kd;
        L.tap += 1;
        if (L.tap == 4u) m_write(L, a, true, normalize(L.g), L.i);
        return;
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
            return;
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
        return;
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
            return;
        }
        L.i += 1;
        if (L.i >= max_steps) m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
        return;
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

template <int TM, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) k_march(const __grid_constant__ WaveArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    LaneTape<TM> LT;
    if constexpr (TM == TM_SMEM) {
        if (!stage_tape(smem, a.job0.tape, a.tape_bytes, a.status)) return;
        LT.T = tape_view(smem);
    } else {
        LT.p = a.job0.tape;
    }
    const uint32_t n = item_count(a);
    MLane L;
    L.item = NIL;
    L.phase = M_IDLE;
    bool retired = false;
    for (;;) {
        bool fresh;
        refill(L.item, retired, n, a.counter, fresh);
        if (__ballot_sync(0xFFFFFFFFu, !retired) == 0u) break;
        if (fresh && !m_start(L, LT, a)) continue;
#pragma unroll 1
        for (int u = 0; u < UNROLL; ++u) {
            if (L.phase == M_IDLE) break;
            m_step(L, LT, a);
        }
    }
}

// ------------------------------------------------------------------------------------------
// ao: Marcher::ambient_occlusion (march.rs:264-280) at every hit
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void ao_slot(const WaveArgs& a, uint32_t slot) {
    uint2 hm = a.b.h_m[slot];
    if (hm.x == NIL) {
        a.b.occ[slot] = 1.0f;
        return;
    }
    const Tape T = tape_view(job_ref(a, slot_job(a, slot)).tape);
    const TapeHeader& h = *T.h;
    uint32_t ns = h.ao_samples;
    // A table of jobs runs AO for every job; the shading of a job without AO ignores it.
    if (ns == 0 || (a.jobs && !(h.flags & SF_AO))) {
        a.b.occ[slot] = 1.0f;
        return;
    }
    float4 hn4 = a.b.h_n[slot], o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
    V hp = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
    V n{hn4.x, hn4.y, hn4.z};
    float base = fmaxf(h.normal_h, 0.01f);
    float span = (float)((ns > 2u ? ns : 2u) - 1u);
    float occ = 0.0f, sca = 1.0f;
    for (uint32_t i = 0; i < ns; ++i) {
        float hr = base + 0.12f * (float)i / span;
        float d = world_eval(T, hp + scale(n, hr)).d;
        occ = occ + (hr - d) * sca;
        sca = sca * 0.92f;
    }
    a.b.occ[slot] = clampf(1.0f - 2.6f * occ, 0.0f, 1.0f);
}

__global__ void __launch_bounds__(SHADE_THREADS) k_ao(const __grid_constant__ WaveArgs a) {
    const uint32_t n = item_count(a);
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n; slot += gridDim.x * blockDim.x)
        ao_slot(a, slot);
}

// ------------------------------------------------------------------------------------------
// shadow: Marcher::soft_shadow (march.rs:227-259) per (hit, light), one march per lane
// ------------------------------------------------------------------------------------------
struct SLane {
    uint32_t item, si;
    V so, sdir;
    float st, sres, sk, smax;
};

template <int TM>
__device__ __forceinline__ bool s_start(SLane& S, LaneTape<TM>& LT, const WaveArgs& a) {
    const uint32_t nl = a.lights_max;
    uint32_t slot = S.item / nl, li = S.item % nl;
    uint2 hm = a.b.h_m[slot];
    if (hm.x != NIL) {
        float4 hn4 = a.b.h_n[slot], o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
        uint32_t job = a.jobs ? __float_as_uint(d4.w) : 0u;
        LT.set(job_ref(a, job).tape);
        const Tape T = LT.get();
        const TapeHeader& h = *T.h;
        if (li < h.n_lights && (h.flags & SF_SHADOWS) && h.shadow_steps > 0) {
            V hp = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
            V hn{hn4.x, hn4.y, hn4.z};
            const DevLight& lt = T.light[li];
            V ldir;
            float ldist;
            light_toward(lt, hp, ldir, ldist);
            if (fmaxf(dot(hn, ldir), 0.0f) > 0.0f) {  // lib.rs:1315-1322
                float lift = fmaxf(h.normal_h * 2.0f, 0.01f);
                S.so = hp + scale(hn, lift);
                S.sdir = ldir;
                S.smax = fminf(ldist, h.max_dist);
                S.sk = light_shadow_k(lt, ldist);
                float hb = S.so.x * 127.1f + S.so.y * 311.7f + S.so.z * 74.7f;
                float sv = sinf(hb) * 43758.547f;
                S.st = 0.02f + fabsf(sv - truncf(sv)) * 0.16f;
                S.sres = 1.0f;
                S.si = 0;
                return true;
            }
        }
    }
    a.b.shadow[S.item] = -1.0f;
    S.item = NIL;
    return false;
}

template <int TM>
__device__ __forceinline__ void s_step(SLane& S, const LaneTape<TM>& LT, const WaveArgs& a) {
    const Tape T = LT.get();
    float hh = world_eval(T, S.so + scale(S.sdir, S.st)).d;
    if (hh < 0.0008f) {
        a.b.shadow[S.item] = 0.0f;
        S.item = NIL;
        return;
    }
    S.sres = fminf(S.sres, S.sk * hh / S.st);
    S.st = S.st + clampf(hh, 0.06f, 0.5f + 0.7f * S.st);
    S.si += 1;
    if (S.st > S.smax || S.si >= T.h->shadow_steps) {
        a.b.shadow[S.item] = clampf(S.sres, 0.0f, 1.0f);
        S.item = NIL;
    }
}

template <int TM, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) k_shadow(const __grid_constant__ WaveArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    LaneTape<TM> LT;
    if constexpr (TM == TM_SMEM) {
        if (!stage_tape(smem, a.job0.tape, a.tape_bytes, a.status)) return;
        LT.T = tape_view(smem);
    } else {
        LT.p = a.job0.tape;
    }
    const uint32_t n = item_count(a) * a.lights_max;
    SLane S;
    S.item = NIL;
    bool retired = false;
    for (;;) {
        bool fresh;
        refill(S.item, retired, n, a.counter, fresh);
        if (__ballot_sync(0xFFFFFFFFu, !retired) == 0u) break;
        if (fresh && !s_start(S, LT, a)) continue;
#pragma unroll 1
        for (int u = 0; u < UNROLL; ++u) {
            if (S.item == NIL) break;
            s_step(S, LT, a);
        }
    }
}

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
    V acc{0.f, 0.f, 0.f};
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
    }
    V o = scale(acc, 1.0f / (float)spp);
    a.b.hdr[(size_t)J.pixel_base + (size_t)y * J.width + x] = make_float4(o.x, o.y, o.z, 1.0f);
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

// Launch-log bracket of one pass.
struct LogScope {
    LaunchLog* l;
    uint32_t kind;
    cudaStream_t s;
    LogScope(LaunchLog* log, uint32_t k, cudaStream_t st, uint32_t n) : l(log), kind(k), s(st) {
        if (l) {
            l->launches += n;
            if (l->begin) l->begin(l->recorder, kind, s);
        }
    }
    ~LogScope() {
        if (l && l->end) l->end(l->recorder, kind, s);
    }
};

typedef void (*WaveKernel)(const WaveArgs);

// Instantiations of a persistent kernel over (tape mode, block, unroll).
struct PersistentSet {
    WaveKernel k[2][2][2];  // [tape mode][block 128 / 256][unroll 1 / 2]
};

#define MM3E_PERSISTENT_SET(K)                                                                     \
    PersistentSet {                                                                                \
        {{{K<TM_SMEM, 128, 1>, K<TM_SMEM, 128, 2>}, {K<TM_SMEM, 256, 1>, K<TM_SMEM, 256, 2>}},     \
         {{K<TM_MULTI, 128, 1>, K<TM_MULTI, 128, 2>}, {K<TM_MULTI, 256, 1>, K<TM_MULTI, 256, 2>}}} \
    }

cudaError_t launch_persistent(const PersistentSet& set, const WaveArgs& a, const TuneParams& t, cudaStream_t s,
                              int sm_count, uint32_t items_per_item) {
    bool use_smem = !a.jobs && a.tape_bytes <= SMEM_TAPE_MAX;
    int bi = t.block >= 256 ? 1 : 0;
    int ui = t.unroll >= 2 ? 1 : 0;
    int block = bi ? 256 : 128;
    WaveKernel k = set.k[use_smem ? 0 : 1][bi][ui];
    size_t smem = use_smem ? a.tape_bytes : 0;
    if (use_smem && smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TAPE_MAX);
        if (e != cudaSuccess) return e;
    }
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
    k<<<blocks, block, smem, s>>>(a);
    return cudaGetLastError();
}

unsigned grid_for(uint64_t n, int threads, uint32_t cap = 0) {
    uint64_t g = (n + threads - 1) / threads;
    if (cap && g > cap) g = cap;
    return g > 0 ? (unsigned)g : 1u;
}

}  // namespace

cudaError_t launch_march(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log) {
    static const PersistentSet set = MM3E_PERSISTENT_SET(k_march);
    LogScope sc(log, KK_MARCH, s, 1);
    return launch_persistent(set, a, t, s, sm_count, 1);
}

cudaError_t launch_shadow(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log) {
    static const PersistentSet set = MM3E_PERSISTENT_SET(k_shadow);
    LogScope sc(log, KK_SHADOW, s, 1);
    return launch_persistent(set, a, t, s, sm_count, a.lights_max ? a.lights_max : 1);
}

// Non-persistent kernels are sized for the largest queue (a.n_items) and read the live count
// from n_items_dev when set.
cudaError_t launch_ao(const WaveArgs& a, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_AO, s, 1);
    k_ao<<<grid_for(a.n_items, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_shade(const WaveArgs& a, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_SHADE, s, 1);
    k_shade<<<grid_for(a.n_items, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a);
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
