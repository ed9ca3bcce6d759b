// engine.cpp — pass-sequence driver, pass buffers and the kernel-time profiler.
#include "engine.h"

#include <utility>

namespace mm3e {

namespace {
template <class T> cudaError_t grow(T** p, size_t n) {
    return cudaMalloc(reinterpret_cast<void**>(p), (n ? n : 1) * sizeof(T) + 16);
}
}  // namespace

void PassBuffers::release() {
    void* ps[] = {qa_o, qa_d, h_n, h_m, occ, shadow, lvl, term, hdr, bright, blur, counters};
    for (void* p : ps) cudaFree(p);
    for (int v = 0; v < MAX_LEVELS; ++v) {
        void* lp[] = {lq_o[v], lq_d[v], lh_n[v], lh_m[v], locc[v], lshadow[v]};
        for (void* p : lp) cudaFree(p);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (aux) cudaStreamDestroy(aux);
    *this = PassBuffers();
}

size_t PassBuffers::bytes_for(size_t cap, size_t lights, size_t levels, size_t pixels) {
    size_t l = lights ? lights : 1, v = levels ? levels : 1;
    // per level: a ray queue (2 float4) and a hit set (float4 + uint2 + AO + a shadow per light)
    return cap * (v * (2 * sizeof(float4) + sizeof(float4) + sizeof(uint2) + sizeof(float) + l * sizeof(float)) +
                  2 * v * sizeof(float4) + sizeof(float4)) +
           pixels * 3 * sizeof(float4) + N_COUNTERS * sizeof(uint32_t);
}

size_t PassBuffers::bytes() const { return cap ? bytes_for(cap, lights, levels, pixels) : 0; }

cudaError_t PassBuffers::ensure(size_t need_cap, size_t need_lights, size_t need_levels, size_t need_pixels) {
    if (counters && need_cap <= cap && need_lights <= lights && need_levels <= levels && need_pixels <= pixels)
        return cudaSuccess;
    size_t c = need_cap > cap ? need_cap : cap;
    size_t l = need_lights > lights ? need_lights : lights;
    size_t v = need_levels > levels ? need_levels : levels;
    size_t px = need_pixels > pixels ? need_pixels : pixels;
    if (v > (size_t)MAX_LEVELS) v = MAX_LEVELS;
    release();
    c = c ? c : 1;
    l = l ? l : 1;
    v = v ? v : 1;
    cudaError_t e;
    if ((e = grow(&qa_o, c)) || (e = grow(&qa_d, c)) || (e = grow(&h_n, c)) || (e = grow(&h_m, c)) ||
        (e = grow(&occ, c)) || (e = grow(&shadow, c * l)) || (e = grow(&lvl, c * 2 * v)) || (e = grow(&term, c)) ||
        (e = grow(&hdr, px)) || (e = grow(&bright, px)) || (e = grow(&blur, px)) ||
        (e = grow(&counters, (size_t)N_COUNTERS))) {
        release();
        return e;
    }
    for (size_t k = 1; k < v; ++k)
        if ((e = grow(&lq_o[k], c)) || (e = grow(&lq_d[k], c)) || (e = grow(&lh_n[k], c)) || (e = grow(&lh_m[k], c)) ||
            (e = grow(&locc[k], c)) || (e = grow(&lshadow[k], c * l))) {
            release();
            return e;
        }
    if (v >= 2 && ((e = cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking)) ||
                   (e = cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming)) ||
                   (e = cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming)))) {
        release();
        return e;
    }
    if ((e = cudaMemset(counters, 0, N_COUNTERS * sizeof(uint32_t))) != cudaSuccess) {
        release();
        return e;
    }
    cap = c;
    lights = l;
    levels = v;
    pixels = px;
    return cudaSuccess;
}

void PreviewBuffers::release() {
    // fields reset one by one: a temporary PreviewBuffers would run this again from its destructor
    void* ps[] = {color, out, depth, obj, keys, filled, hole_pix, count, mover, delta};
    for (void* p : ps) cudaFree(p);
    color = out = nullptr;
    depth = nullptr;
    obj = nullptr;
    keys = nullptr;
    filled = nullptr;
    hole_pix = count = nullptr;
    mover = nullptr;
    delta = nullptr;
    pixels = movers = deltas = 0;
}

size_t PreviewBuffers::bytes() const {
    return pixels * (2 * sizeof(uchar4) + sizeof(float) + sizeof(int32_t) + sizeof(unsigned long long) + 1 +
                     sizeof(uint32_t)) +
           movers * sizeof(float4) + deltas * 3 * sizeof(float) + sizeof(uint32_t);
}

cudaError_t PreviewBuffers::ensure(size_t need_pixels, size_t need_movers, size_t need_deltas) {
    if (count && need_pixels <= pixels && need_movers <= movers && need_deltas <= deltas) return cudaSuccess;
    size_t n = need_pixels > pixels ? need_pixels : pixels;
    size_t m = need_movers > movers ? need_movers : movers;
    size_t d = need_deltas > deltas ? need_deltas : deltas;
    n = n ? n : 1;
    m = m > 8 ? m : 8;
    d = d > 8 ? d : 8;
    release();
    cudaError_t e;
    if ((e = grow(&color, n)) || (e = grow(&out, n)) || (e = grow(&depth, n)) || (e = grow(&obj, n)) ||
        (e = grow(&keys, n)) || (e = grow(&filled, n)) || (e = grow(&hole_pix, n)) || (e = grow(&count, 1)) ||
        (e = grow(&mover, m)) || (e = grow(&delta, 3 * d))) {
        release();
        return e;
    }
    pixels = n;
    movers = m;
    deltas = d;
    return cudaSuccess;
}

// ---------------------------------------------------------------------------------------
Profiler::~Profiler() {
    for (cudaEvent_t e : pool_) cudaEventDestroy(e);
}

cudaEvent_t Profiler::event() {
    if (used_ == pool_.size()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        pool_.push_back(e);
    }
    return pool_[used_++];
}

void Profiler::begin(uint32_t kind, cudaStream_t s) {
    (void)kind;
    cudaEvent_t e = event();
    if (e) cudaEventRecord(e, s);
    open_.push_back(e);
}

void Profiler::end(uint32_t kind, cudaStream_t s) {
    if (open_.empty()) return;
    cudaEvent_t a = open_.back();
    open_.pop_back();
    cudaEvent_t b = event();
    if (!a || !b) return;
    cudaEventRecord(b, s);
    recs_.push_back(Rec{kind, a, b});
}

cudaError_t Profiler::collect(double* ms, uint32_t* launches) {
    cudaError_t err = cudaSuccess;
    for (const Rec& r : recs_) {
        cudaError_t e = cudaEventSynchronize(r.b);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.a, r.b);
        if (e != cudaSuccess) {
            err = e;
            continue;
        }
        if (r.kind < KK_COUNT) {
            ms[r.kind] += t;
            launches[r.kind] += 1;
        }
    }
    recs_.clear();
    open_.clear();
    used_ = 0;
    return err;
}

namespace {
void prof_begin(void* p, uint32_t k, cudaStream_t s) { static_cast<Profiler*>(p)->begin(k, s); }
void prof_end(void* p, uint32_t k, cudaStream_t s) { static_cast<Profiler*>(p)->end(k, s); }
}  // namespace

LaunchLog Profiler::log() {
    LaunchLog l;
    if (on) {
        l.recorder = this;
        l.begin = prof_begin;
        l.end = prof_end;
    }
    return l;
}

// ---------------------------------------------------------------------------------------
namespace {
WaveArgs wave_args(const PassPlan& plan, PassBuffers& buf, const TuneParams& tune, int sm_count) {
    WaveArgs a{};
    a.job0 = plan.job0;
    a.jobs = plan.jobs;
    a.totals = plan.totals;
    a.n_jobs = 1;
    a.tape_bytes = plan.tape_bytes;
    a.cap = (uint32_t)buf.cap;
    a.lights_max = plan.lights_max;
    a.tile_wlog = tune.tile_wlog;
    a.grid_cap = (uint32_t)sm_count * 16u;
    a.status = buf.counters + (N_COUNTERS - 1);
    a.b.q_o = buf.qa_o;
    a.b.q_d = buf.qa_d;
    a.b.h_n = buf.h_n;
    a.b.h_m = buf.h_m;
    a.b.occ = buf.occ;
    a.b.shadow = buf.shadow;
    a.b.lvl = buf.lvl;
    a.b.term = buf.term;
    a.b.hdr = buf.hdr;
    a.b.fg = buf.bright;
    a.film = plan.film ? 1u : 0u;
    for (int k = 1; k < MAX_LEVELS && k < (int)buf.levels; ++k) {
        a.lq_o[k] = buf.lq_o[k];
        a.lq_d[k] = buf.lq_d[k];
        a.lh_n[k] = buf.lh_n[k];
        a.lh_m[k] = buf.lh_m[k];
        a.lq_count[k] = buf.counters + 4 * (k - 1) + 2;
    }
    return a;
}
}  // namespace

namespace {
const uint32_t* primary_count(const PassPlan& plan) {
    if (plan.queue0) return plan.queue0;
    return plan.jobs ? &plan.totals->n_samples : nullptr;
}

// The AO, shadow and shading passes of one level whose hits exist (queue / hit set in a.b).
cudaError_t shade_passes(const PassPlan& plan, WaveArgs& a, PassBuffers& buf, const TuneParams& tune, cudaStream_t s,
                         int sm_count, LaunchLog* log, uint32_t level) {
    cudaError_t e;
    a.level = level;
    a.src = level == 0 && !plan.queue0 ? SRC_SAMPLES : SRC_QUEUE;
    a.n_items = plan.n_samples;
    a.n_items_dev = level == 0 ? primary_count(plan) : buf.counters + 4 * (level - 1) + 2;
    a.chain_levels = 0;
    if (plan.ao && (e = launch_ao(a, s, log, plan.spec)) != cudaSuccess) return e;
    if (plan.shadows && plan.lights_max > 0) {
        a.counter = buf.counters + 4 * level + 1;
        if ((e = launch_shadow(a, tune, s, sm_count, log, plan.spec)) != cudaSuccess) return e;
    }
    return launch_shade(a, s, log);
}

// One level on its own (no reflections): march, then AO, shadows and shading.
cudaError_t level_passes(const PassPlan& plan, WaveArgs& a, PassBuffers& buf, const TuneParams& tune, cudaStream_t s,
                         int sm_count, LaunchLog* log, uint32_t level) {
    cudaError_t e;
    a.level = level;
    a.src = level == 0 && !plan.queue0 ? SRC_SAMPLES : SRC_QUEUE;
    a.n_items = plan.n_samples;
    a.n_items_dev = level == 0 ? primary_count(plan) : buf.counters + 4 * (level - 1) + 2;
    a.counter = buf.counters + 4 * level;
    a.chain_levels = 0;
    if ((e = launch_march(a, tune, s, sm_count, log, plan.spec)) != cudaSuccess) return e;
    return shade_passes(plan, a, buf, tune, s, sm_count, log, level);
}
}  // namespace

cudaError_t run_beauty(const PassPlan& plan, PassBuffers& buf, const TuneParams& tune, cudaStream_t s, int sm_count,
                       LaunchLog* log) {
    cudaError_t e = cudaMemsetAsync(buf.counters, 0, (N_COUNTERS - (plan.clear_status ? 0 : 1)) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    WaveArgs a = wave_args(plan, buf, tune, sm_count);
    const uint32_t levels = plan.levels > buf.levels ? (uint32_t)buf.levels : plan.levels;
    if (levels <= 1) {
        if ((e = level_passes(plan, a, buf, tune, s, sm_count, log, 0)) != cudaSuccess) return e;
    } else {
        // the primary march runs every reflection chain too; then the levels shade side by side
        WaveArgs a0 = a;
        a0.level = 0;
        a0.src = plan.queue0 ? SRC_QUEUE : SRC_SAMPLES;
        a0.n_items = plan.n_samples;
        a0.n_items_dev = primary_count(plan);
        a0.counter = buf.counters;
        a0.chain_levels = levels;
        if ((e = launch_march(a0, tune, s, sm_count, log, plan.spec)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(buf.ev_fork, s)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(buf.aux, buf.ev_fork, 0)) != cudaSuccess) return e;
        for (uint32_t level = 1; level < levels; ++level) {
            WaveArgs ak = a;
            ak.b.q_o = buf.lq_o[level];
            ak.b.q_d = buf.lq_d[level];
            ak.b.h_n = buf.lh_n[level];
            ak.b.h_m = buf.lh_m[level];
            ak.b.occ = buf.locc[level];
            ak.b.shadow = buf.lshadow[level];
            if ((e = shade_passes(plan, ak, buf, tune, buf.aux, sm_count, log, level)) != cudaSuccess) return e;
        }
        if ((e = cudaEventRecord(buf.ev_join, buf.aux)) != cudaSuccess) return e;
        if ((e = shade_passes(plan, a0, buf, tune, s, sm_count, log, 0)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(s, buf.ev_join, 0)) != cudaSuccess) return e;
    }
    if (plan.queue0) return cudaSuccess;
    if ((e = launch_resolve(a, plan.n_slots, s, log)) != cudaSuccess) return e;
    if (!plan.post) return cudaSuccess;
    return run_post(plan, buf, s, sm_count, log);
}

cudaError_t run_post(const PassPlan& plan, PassBuffers& buf, cudaStream_t s, int sm_count, LaunchLog* log) {
    PostArgs p{};
    p.job0 = plan.job0;
    p.jobs = plan.jobs;
    p.totals = plan.totals;
    p.n_jobs = 1;
    p.n_pixels = plan.n_pixels;
    p.any_bloom = plan.bloom ? 1 : 0;
    p.grid_cap = (uint32_t)sm_count * 16u;
    p.hdr = buf.hdr;
    p.bright = buf.bright;
    p.blur_h = buf.blur;
    return launch_post(p, s, log);
}

}  // namespace mm3e
