// march_kernels.cuh — bodies of the persistent march and soft-shadow passes and the AO pass,
// templated on the field evaluation: the library instantiates them with the tape interpreter
// (InterpField); a scene-specialised program compiled at run time with NVRTC instantiates them
// with its generated field (the same device functions with the scene's records folded in).
//
// The march and shadow passes are persistent: every lane runs one ray at a time, one field
// sample per loop iteration (or `UNROLL` samples between refills); a lane that finishes
// refills from a global counter with one warp-aggregated atomic (ballot + popc + shfl), so
// warps stay full without a separate compaction pass. With a single job whose tape fits, each
// CTA first stages the tape into shared memory with TMA bulk copies (cp.async.bulk) completing
// on an mbarrier; with many jobs every lane reads its ray's job's tape through the L1 cache.
#pragma once
#include "device_math.cuh"
#include "kernels.h"

namespace mm3e {
namespace wave {

// The tape interpreter's world field (WorldPlan::eval, accel.rs:209-252), the marcher settings
// read from the tape header, and the exact-gradient normal over the tape's objects. A
// scene-specialised program supplies a class with the same members that returns its scene's
// settings as constants, so the pass bodies fold their branches on them.
struct InterpField {
    static constexpr bool kConstSettings = false;  // the settings below are read at run time
    static __device__ __forceinline__ Field eval(const Tape& T, V p) { return world_eval(T, p); }
    static __device__ __forceinline__ V normal_dual(const Tape& T, V p) {
        return mm3e::normal_dual(T.obj, T.h->n_objects, p);
    }
    static __device__ __forceinline__ uint32_t flags(const TapeHeader& h) { return h.flags; }
    static __device__ __forceinline__ uint32_t max_steps(const TapeHeader& h) { return h.max_steps; }
    static __device__ __forceinline__ uint32_t shadow_steps(const TapeHeader& h) { return h.shadow_steps; }
    static __device__ __forceinline__ uint32_t ao_samples(const TapeHeader& h) { return h.ao_samples; }
    static __device__ __forceinline__ uint32_t n_lights(const TapeHeader& h) { return h.n_lights; }
    static __device__ __forceinline__ float max_dist(const TapeHeader& h) { return h.max_dist; }
    static __device__ __forceinline__ float eps(const TapeHeader& h) { return h.eps; }
    static __device__ __forceinline__ float step_scale(const TapeHeader& h) { return h.step_scale; }
    static __device__ __forceinline__ float lod_footprint(const TapeHeader& h) { return h.lod_footprint; }
    static __device__ __forceinline__ float subitize(const TapeHeader& h) { return h.subitize; }
    static __device__ __forceinline__ float normal_h(const TapeHeader& h) { return h.normal_h; }
};


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

// Whether an earlier pass of this call gave up (its tape staging timed out or found a corrupt
// tape): the passes after it then do nothing, since the hit records they would read were never
// written, and the call reports the error. The word is constant while a pass runs (only earlier
// launches in stream order write it), so the early return is uniform.
__device__ __forceinline__ bool pass_failed(const WaveArgs& a) {
    return a.status && (*(volatile const uint32_t*)a.status & (ST_TAPE_TIMEOUT | ST_TAPE_CORRUPT)) != 0u;
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
// mbarrier, waited on with an iteration limit (`limit`, 0: 2^22). Returns false (status word
// set) on failure. A wait that gives up while copies were issued waits again, with a longer
// limit, for them to land, so the CTA does not return with a copy still writing its shared
// memory. With `probe` nothing arrives on the barrier and no copy is issued: the wait runs to
// its limit with nothing in flight (a test of the give-up path).
__device__ __forceinline__ bool stage_tape(unsigned char* smem, const unsigned char* tape, uint32_t bytes,
                                           uint32_t* status, uint32_t limit, bool probe) {
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
    if (threadIdx.x == 0 && !probe) {
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
    if (!mbar_wait(mbar, 0u, limit ? limit : (1u << 22))) {
        tape_ok = 0u;
        if (!probe) mbar_wait(mbar, 0u, 1u << 26);  // the issued copies land before the CTA leaves
    }
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

// film.rs:218-224
__device__ __forceinline__ uint32_t film_hash(uint32_t v) {
    v ^= v >> 16;
    v *= 0x7feb352du;
    v ^= v >> 15;
    v *= 0x846ca68bu;
    return v ^ (v >> 16);
}

// Thin-lens ray of AA sample (sx, sy) of pixel (x, y): film.rs:199-215's jittered aperture cell,
// camera.rs:92-102's concentric disk and camera.rs:71-90's focus-plane ray; `rd` holds the
// pinhole direction through the image sample on entry.
__device__ __forceinline__ void lens_ray(const FrameJob& J, uint32_t x, uint32_t y, uint32_t sx, uint32_t sy,
                                         uint32_t n, V& ro, V& rd) {
    uint32_t pixel_seed = film_hash(x ^ film_hash(y));
    uint64_t n64 = n;
    uint32_t cell_x = (uint32_t)(((uint64_t)sx + sy + pixel_seed) % n64);
    uint32_t cell_y = (uint32_t)(((uint64_t)sx + 2ull * sy + film_hash(pixel_seed)) % n64);
    uint32_t seed = film_hash(pixel_seed ^ film_hash(sx) ^ film_hash(sy + 0xa511e9b3u));
    float nf = (float)n;
    float u = ((float)cell_x + (float)(seed >> 8) * (1.0f / 16777216.0f)) / nf;
    float v = ((float)cell_y + (float)(film_hash(seed) >> 8) * (1.0f / 16777216.0f)) / nf;
    float px = 2.0f * u - 1.0f, py = 2.0f * v - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (!(px == 0.0f && py == 0.0f)) {
        float radius, theta;
        if (fabsf(px) > fabsf(py)) {
            radius = px;
            theta = 0.785398163397448309616f * (py / px);
        } else {
            radius = py;
            theta = 1.57079632679489661923f - 0.785398163397448309616f * (px / py);
        }
        dx = radius * cosf(theta);
        dy = radius * sinf(theta);
    }
    float r = J.lens_radius;
    V eye = ld3(J.cam.eye);
    V origin = eye + scale(ld3(J.cam.right), dx * r) + scale(ld3(J.cam.up), dy * r);
    V focus = eye + scale(rd, J.focus_distance / dot(rd, ld3(J.cam.fwd)));
    ro = origin;
    rd = normalize(focus - origin);
}

// Which boosts of Marcher::march_with a scene's settings allow (march.rs:132-141): over-
// relaxation (omega 1.4, relaxed to 1 after a rollback) only with step_scale >= 1, the leap only
// with a positive subitize as well, the secant step only with the secant flag as well. A field
// class with constant settings (a scene-specialised program) turns a boost that cannot occur
// into a compile-time false, and its lane state is never read or kept; the interpreter keeps all.
template <class FP> struct MarchBoosts {
    bool relax, leap, secant;
    __device__ __forceinline__ explicit MarchBoosts(const TapeHeader& h) {
        const bool lip = FP::step_scale(h) >= 1.0f;
        relax = !FP::kConstSettings || lip;
        leap = !FP::kConstSettings || (lip && FP::subitize(h) > 0.0f);
        secant = !FP::kConstSettings || (lip && (FP::flags(h) & SF_SECANT) != 0u);
    }
};

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
    uint32_t hmat;
    // Phase scratch, never needed by two phases at once: M_COVER keeps the step's distance,
    // radius and epsilon in x0..x2 and its material in xu; M_TETRA keeps the gradient sum in
    // x0..x2 and the tap index in xu.
    float x0, x1, x2;
    uint32_t xu;
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
template <int TM, class FP>
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
        if (inside && aa > 1u && J.lens_radius > 0.0f) lens_ray(J, x, y, sx, sy, aa, L.ro, L.rd);
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
    const MarchBoosts<FP> can(h);
    bool lip = FP::step_scale(h) >= 1.0f;
    if (can.secant) L.d_prev = __int_as_float(0x7f800000);
    if (can.relax) L.omega = lip ? 1.4f : FP::step_scale(h);
    if (can.leap) L.subz = lip ? FP::subitize(h) : 0.0f;
    if (can.secant) L.secant_on = ((FP::flags(h) & SF_SECANT) && lip) ? 1u : 0u;
    if (can.leap || can.secant) L.boost = BOOST_OMEGA;
    L.i = 0;
    L.phase = M_MARCH;
    if (FP::max_steps(h) == 0) {
        m_write(L, a, false, V{0.f, 0.f, 0.f}, 0u);
        return false;
    }
    return true;
}

// One field sample of the lane's ray and the state transition it causes.
template <int TM, class FP>
__device__ __forceinline__ void m_step(MLane& L, const LaneTape<TM>& LT, const WaveArgs& a) {
    const Tape T = LT.get();
    const TapeHeader& h = *T.h;
    const uint32_t max_steps = FP::max_steps(h);
    V p;
    if (L.phase == M_MARCH) p = m_at(L, L.t);
    else if (L.phase == M_COVER) p = m_at(L, 0.5f * ((L.t_prev + L.prev_r) + (L.t - L.x1)));
    else p = m_at(L, L.t) + scale(tetra_k(L.xu), FP::normal_h(h));
    Field f = FP::eval(T, p);
    if (L.phase == M_TETRA) {
        V kd = scale(tetra_k(L.xu), f.d);
        V g = L.xu == 0 ? kd : V{L.x0, L.x1, L.x2} + kd;
        L.x0 = g.x;
        L.x1 = g.y;
        L.x2 = g.z;
        L.xu += 1;
        if (L.xu == 4u) m_write(L, a, true, normalize(g), L.i);
        return;
    }
    float d;
    uint32_t m;
    float radius, e;
    if (L.phase == M_MARCH) {
        d = f.d;
        m = f.m;
        radius = fabsf(d);
        // With a zero footprint, lod * t is a zero for every finite t (t is finite here: it
        // passed the max_dist test). Adding a zero leaves a nonzero sum as it is and can change
        // only the sign of a zero one, and e enters nothing but comparisons, where that sign does
        // not count; so a field class with constant settings leaves the term out.
        if (FP::kConstSettings && FP::lod_footprint(h) == 0.0f) e = FP::eps(h) * (1.0f + L.t * 0.5f);
        else e = FP::eps(h) * (1.0f + L.t * 0.5f) + FP::lod_footprint(h) * L.t;
        // With a step scale in [0, 1) there is no boost, so a step is fl(d_prev * scale), at most
        // |d_prev| = prev_r (and 0 after a rollback): it never exceeds radius + prev_r, and with
        // constant settings that test and the COVER phase it leads to are compiled out.
        const bool can_overshoot = !FP::kConstSettings || !(FP::step_scale(h) >= 0.0f && FP::step_scale(h) < 1.0f);
        bool overlap_fail = (L.step > 0.0f && d < 0.0f) || (can_overshoot && L.step > radius + L.prev_r);
        if (overlap_fail && d > 0.0f) {  // check the gap midpoint first
            L.x0 = d;
            L.xu = m;
            L.x1 = radius;
            L.x2 = e;
            L.phase = M_COVER;
            return;
        }
        if (overlap_fail) goto rollback;
    } else {  // M_COVER
        float gap_lo = L.t_prev + L.prev_r;
        float gap_hi = L.t - L.x1;
        L.phase = M_MARCH;
        if (!(f.d >= 0.5f * (gap_hi - gap_lo))) goto rollback;
        d = L.x0;
        m = L.xu;
        radius = L.x1;
        e = L.x2;
    }
    // march.rs:173-206
    if (d < e) {
        L.hmat = m;
        if (FP::flags(h) & SF_DUAL_SAFE) {
            m_write(L, a, true, FP::normal_dual(T, m_at(L, L.t)), L.i);
        } else {
            L.phase = M_TETRA;
            L.xu = 0;
        }
        return;
    }
    {
        const MarchBoosts<FP> can(h);
        float step_len = d * (can.relax ? L.omega : FP::step_scale(h));
        uint32_t boost = BOOST_OMEGA;
        if (can.leap && L.subz > 0.0f && d > e * 6.0f) {
            step_len = step_len * (1.0f + L.subz);
            boost = BOOST_LEAP;
        }
        if (can.secant && L.secant_on && d < 0.08f && isfinite(L.d_prev)) {
            float dt = L.t - L.t_prev;
            float dd = d - L.d_prev;
            if (dt > 1e-6f && dd < -1e-6f) {
                step_len = clampf(-d * dt / dd, d, d * 4.0f);
                boost = BOOST_SECANT;
            }
        }
        L.step = step_len;
        if (can.leap || can.secant) L.boost = boost;
        L.prev_r = radius;
        if (can.secant) L.d_prev = d;
        L.t_prev = L.t;
        L.t = L.t + step_len;
        if (L.t > FP::max_dist(h)) {
            m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
            return;
        }
        L.i += 1;
        if (L.i >= max_steps) m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
        return;
    }
rollback:  // retreat to the last safe frontier (march.rs:155-170)
    L.t = L.t_prev + L.prev_r;
    {
        const MarchBoosts<FP> can(h);
        const uint32_t boost = (can.leap || can.secant) ? L.boost : (uint32_t)BOOST_OMEGA;
        if (boost == BOOST_OMEGA) {
            if (can.relax) L.omega = fminf(L.omega, 1.0f);  // (step_scale < 1 stays as it is)
        } else if (boost == BOOST_LEAP) {
            L.subz = 0.0f;
        } else {
            L.secant_on = 0;
        }
        if (can.leap || can.secant) L.boost = BOOST_OMEGA;
        if (can.secant) L.d_prev = __int_as_float(0x7f800000);
    }
    L.prev_r = 0.0f;
    L.step = 0.0f;
    L.i += 1;
    if (L.i >= max_steps) m_write(L, a, false, V{0.f, 0.f, 0.f}, max_steps);
}

template <int TM, int UNROLL, class FP>
__device__ __forceinline__ void march_body(const WaveArgs& a) {
    extern __shared__ __align__(128) unsigned char smem[];
    LaneTape<TM> LT;
    if constexpr (TM == TM_SMEM) {
        if (!stage_tape(smem, a.job0.tape, a.tape_bytes, a.status, a.wait_limit, a.wait_probe != 0u)) return;
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
        if (fresh && !m_start<TM, FP>(L, LT, a)) continue;
#pragma unroll 1
        for (int u = 0; u < UNROLL; ++u) {
            if (L.phase == M_IDLE) break;
            m_step<TM, FP>(L, LT, a);
        }
    }
}

// ------------------------------------------------------------------------------------------
// ao: Marcher::ambient_occlusion (march.rs:264-280) at every hit
// ------------------------------------------------------------------------------------------
template <class FP>
__device__ __forceinline__ void ao_slot(const WaveArgs& a, uint32_t slot) {
    uint2 hm = a.b.h_m[slot];
    if (hm.x == NIL) {
        a.b.occ[slot] = 1.0f;
        return;
    }
    const Tape T = tape_view(job_ref(a, slot_job(a, slot)).tape);
    const TapeHeader& h = *T.h;
    uint32_t ns = FP::ao_samples(h);
    // A table of jobs runs AO for every job; the shading of a job without AO ignores it.
    if (ns == 0 || (a.jobs && !(FP::flags(h) & SF_AO))) {
        a.b.occ[slot] = 1.0f;
        return;
    }
    float4 hn4 = a.b.h_n[slot], o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
    V hp = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
    V n{hn4.x, hn4.y, hn4.z};
    float base = fmaxf(FP::normal_h(h), 0.01f);
    float span = (float)((ns > 2u ? ns : 2u) - 1u);
    float occ = 0.0f, sca = 1.0f;
    for (uint32_t i = 0; i < ns; ++i) {
        float hr = base + 0.12f * (float)i / span;
        float d = FP::eval(T, hp + scale(n, hr)).d;
        occ = occ + (hr - d) * sca;
        sca = sca * 0.92f;
    }
    a.b.occ[slot] = clampf(1.0f - 2.6f * occ, 0.0f, 1.0f);
}

template <class FP>
__device__ __forceinline__ void ao_body(const WaveArgs& a) {
    if (pass_failed(a)) return;
    const uint32_t n = item_count(a);
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n; slot += gridDim.x * blockDim.x)
        ao_slot<FP>(a, slot);
}

// ------------------------------------------------------------------------------------------
// shadow: Marcher::soft_shadow (march.rs:227-259) per (hit, light), one march per lane
// ------------------------------------------------------------------------------------------
struct SLane {
    uint32_t item, si;
    V so, sdir;
    float st, sres, sk, smax;
};

template <int TM, class FP>
__device__ __forceinline__ bool s_start(SLane& S, LaneTape<TM>& LT, const WaveArgs& a, uint32_t n_slots) {
    // Work items run light-major (all hits' rays toward light 0, then light 1, ...), so a warp's
    // rays share a direction and pass the same objects; results keep the slot-major layout.
    const uint32_t nl = a.lights_max;
    const uint32_t li = S.item / n_slots, slot = S.item - li * n_slots;
    S.item = slot * nl + li;
    uint2 hm = a.b.h_m[slot];
    if (hm.x != NIL) {
        float4 hn4 = a.b.h_n[slot], o4 = a.b.q_o[slot], d4 = a.b.q_d[slot];
        uint32_t job = a.jobs ? __float_as_uint(d4.w) : 0u;
        LT.set(job_ref(a, job).tape);
        const Tape T = LT.get();
        const TapeHeader& h = *T.h;
        if (li < FP::n_lights(h) && (FP::flags(h) & SF_SHADOWS) && FP::shadow_steps(h) > 0) {
            V hp = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
            V hn{hn4.x, hn4.y, hn4.z};
            const DevLight& lt = T.light[li];
            V ldir;
            float ldist;
            light_toward(lt, hp, ldir, ldist);
            if (fmaxf(dot(hn, ldir), 0.0f) > 0.0f) {  // lib.rs:1315-1322
                float lift = fmaxf(FP::normal_h(h) * 2.0f, 0.01f);
                S.so = hp + scale(hn, lift);
                S.sdir = ldir;
                S.smax = fminf(ldist, FP::max_dist(h));
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

template <int TM, class FP>
__device__ __forceinline__ void s_step(SLane& S, const LaneTape<TM>& LT, const WaveArgs& a) {
    const Tape T = LT.get();
    float hh = FP::eval(T, S.so + scale(S.sdir, S.st)).d;
    if (hh < 0.0008f) {
        a.b.shadow[S.item] = 0.0f;
        S.item = NIL;
        return;
    }
    // res = min(res, k*h/t) (march.rs:246). All terms are positive here (h >= 8e-4, k, t > 0), so
    // where k*h exceeds res*t by a relative 2^-20 the quotient cannot undercut res and the
    // division (several instructions in IEEE binary32) is skipped; elsewhere it is taken exactly.
    const float kh = S.sk * hh;
    if (!(kh > S.sres * S.st * 1.00000095f)) S.sres = fminf(S.sres, kh / S.st);
    S.st = S.st + clampf(hh, 0.06f, 0.5f + 0.7f * S.st);
    S.si += 1;
    if (S.st > S.smax || S.si >= FP::shadow_steps(*T.h)) {
        a.b.shadow[S.item] = clampf(S.sres, 0.0f, 1.0f);
        S.item = NIL;
    }
}

template <int TM, int UNROLL, class FP>
__device__ __forceinline__ void shadow_body(const WaveArgs& a) {
    extern __shared__ __align__(128) unsigned char smem[];
    if (pass_failed(a)) return;
    LaneTape<TM> LT;
    if constexpr (TM == TM_SMEM) {
        if (!stage_tape(smem, a.job0.tape, a.tape_bytes, a.status, a.wait_limit, a.wait_probe != 0u)) return;
        LT.T = tape_view(smem);
    } else {
        LT.p = a.job0.tape;
    }
    const uint32_t n_slots = item_count(a);
    const uint32_t n = n_slots * a.lights_max;
    SLane S;
    S.item = NIL;
    bool retired = false;
    for (;;) {
        bool fresh;
        refill(S.item, retired, n, a.counter, fresh);
        if (__ballot_sync(0xFFFFFFFFu, !retired) == 0u) break;
        if (fresh && !s_start<TM, FP>(S, LT, a, n_slots)) continue;
#pragma unroll 1
        for (int u = 0; u < UNROLL; ++u) {
            if (S.item == NIL) break;
            s_step<TM, FP>(S, LT, a);
        }
    }
}

}  // namespace wave
}  // namespace mm3e
