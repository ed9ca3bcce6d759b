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
    void* ps[] = {qa_o, qa_d, qb_o, qb_d, qc_o, qc_d, qd_o, qd_d, h_n, h_m, occ, shadow, h_n1, h_m1, occ1, shadow1,
                  h_n2, h_m2, occ2, shadow2, lvl, term, hdr, fg, blur, counters};
    for (void* p : ps) cudaFree(p);
    if (ev_fork) cudaEventDestroy(ev_fork);
    for (int i = 0; i < MAX_LEVELS; ++i) {
        if (ev_marched[i]) cudaEventDestroy(ev_marched[i]);
        if (ev_shaded[i]) cudaEventDestroy(ev_shaded[i]);
    }
    if (aux) cudaStreamDestroy(aux);
    if (aux2) cudaStreamDestroy(aux2);
    *this = PassBuffers();
}

size_t PassBuffers::bytes_for(size_t cap, size_t lights, size_t levels, size_t pixels) {
    size_t l = lights ? lights : 1, v = levels ? levels : 1;
    size_t queues = v >= 4 ? 8 : (v >= 3 ? 6 : 4), hit_sets = v >= 3 ? 3 : (v >= 2 ? 2 : 1);
    return cap * (queues * sizeof(float4) + hit_sets * (sizeof(float4) + sizeof(uint2) + sizeof(float) +
                                                         l * sizeof(float)) +
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
    release();
    c = c ? c : 1;
    cudaError_t e;
    if ((e = grow(&qa_o, c)) || (e = grow(&qa_d, c)) || (e = grow(&qb_o, c)) || (e = grow(&qb_d, c)) ||
        (e = grow(&h_n, c)) || (e = grow(&h_m, c)) || (e = grow(&occ, c)) || (e = grow(&shadow, c * (l ? l : 1))) ||
        (e = grow(&lvl, c * 2 * (v ? v : 1))) || (e = grow(&term, c)) || (e = grow(&hdr, px)) ||
        (e = grow(&fg, px)) || (e = grow(&blur, px)) || (e = grow(&counters, (size_t)N_COUNTERS))) {
        release();
        return e;
    }
    if (v >= 2 && ((e = grow(&h_n1, c)) || (e = grow(&h_m1, c)) || (e = grow(&occ1, c)) ||
                   (e = grow(&shadow1, c * (l ? l : 1))) ||
                   (e = cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking)) ||
                   (e = cudaStreamCreateWithFlags(&aux2, cudaStreamNonBlocking)) ||
                   (e = cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming)))) {
        release();
        return e;
    }
    for (size_t i = 1; i < v && i < (size_t)MAX_LEVELS; ++i)
        if ((e = cudaEventCreateWithFlags(&ev_marched[i], cudaEventDisableTiming)) ||
            (e = cudaEventCreateWithFlags(&ev_shaded[i], cudaEventDisableTiming))) {
            release();
            return e;
        }
    if (v >= 3 && ((e = grow(&qc_o, c)) || (e = grow(&qc_d, c)) || (e = grow(&h_n2, c)) || (e = grow(&h_m2, c)) ||
                   (e = grow(&occ2, c)) || (e = grow(&shadow2, c * (l ? l : 1))))) {
        release();
        return e;
    }
    if (v >= 4 && ((e = grow(&qd_o, c)) || (e = grow(&qd_d, c)))) {
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
    a.b.nq_o = buf.qb_o;
    a.b.nq_d = buf.qb_d;
    a.b.lvl = buf.lvl;
    a.b.term = buf.term;
    a.b.hdr = buf.hdr;
    a.b.fg = buf.fg;
    a.film = plan.film ? 1u : 0u;
    a.wait_limit = plan.wait_limit;
    a.wait_probe = plan.wait_probe;
    return a;
}
}  // namespace

namespace {
const uint32_t* primary_count(const PassPlan& plan) {
    if (plan.queue0) return plan.queue0;
    return plan.jobs ? &plan.totals->n_samples : nullptr;
}

// The passes of one level: march, AO, shadows, (reflection rays of the next level), shading.
cudaError_t level_passes(const PassPlan& plan, WaveArgs& a, PassBuffers& buf, const TuneParams& tune, cudaStream_t s,
                         int sm_count, LaunchLog* log, uint32_t level, bool reflect_next) {
    cudaError_t e;
    a.level = level;
    a.src = level == 0 && !plan.queue0 ? SRC_SAMPLES : SRC_QUEUE;
    a.n_items = plan.n_samples;
    a.n_items_dev = level == 0 ? primary_count(plan) : buf.counters + 4 * (level - 1) + 2;
    a.b.nq_count = buf.counters + 4 * level + 2;
    a.counter = buf.counters + 4 * level;
    if ((e = launch_march(a, tune, s, sm_count, log, plan.spec)) != cudaSuccess) return e;
    if (reflect_next && (e = launch_reflect(a, s, log)) != cudaSuccess) return e;
    if (plan.ao && (e = launch_ao(a, s, log, plan.spec)) != cudaSuccess) return e;
    if (plan.shadows && plan.lights_max > 0) {
        a.counter = buf.counters + 4 * level + 1;
        if ((e = launch_shadow(a, tune, s, sm_count, log, plan.spec)) != cudaSuccess) return e;
    }
    return launch_shade(a, s, log);
}
}  // namespace

cudaError_t run_beauty(const PassPlan& plan, PassBuffers& buf, const TuneParams& tune, cudaStream_t s, int sm_count,
                       LaunchLog* log) {
    cudaError_t e = cudaMemsetAsync(buf.counters, 0, (N_COUNTERS - (plan.clear_status ? 0 : 1)) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    WaveArgs a = wave_args(plan, buf, tune, sm_count);
    a.emit = 0;  // reflection rays come from the reflect pass, right after each level's march
    const uint32_t levels = plan.levels > buf.levels ? (uint32_t)buf.levels : plan.levels;
    if (levels <= 1) {
        if ((e = level_passes(plan, a, buf, tune, s, sm_count, log, 0, false)) != cudaSuccess) return e;
    } else {
        // primary level on `s`; its reflection rays fork the deeper levels onto the aux streams
        WaveArgs a0 = a;
        a0.b.nq_o = buf.qb_o;
        a0.b.nq_d = buf.qb_d;
        a0.level = 0;
        a0.src = plan.queue0 ? SRC_QUEUE : SRC_SAMPLES;
        a0.n_items = plan.n_samples;
        a0.n_items_dev = primary_count(plan);
        a0.b.nq_count = buf.counters + 2;
        a0.counter = buf.counters;
        if ((e = launch_march(a0, tune, s, sm_count, log, plan.spec)) != cudaSuccess) return e;
        if ((e = launch_reflect(a0, s, log)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(buf.ev_fork, s)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(buf.aux, buf.ev_fork, 0)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(buf.aux2, buf.ev_fork, 0)) != cudaSuccess) return e;
        float4* q_o[3] = {buf.qb_o, buf.qc_o, buf.qd_o};
        float4* q_d[3] = {buf.qb_d, buf.qc_d, buf.qd_d};
        for (uint32_t level = 1; level < levels; ++level) {
            WaveArgs ak = a;
            const uint32_t qi = (level - 1) % 3, ni = level % 3;
            const bool odd = (level & 1u) != 0;
            ak.b.q_o = q_o[qi];
            ak.b.q_d = q_d[qi];
            ak.b.nq_o = q_o[ni];
            ak.b.nq_d = q_d[ni];
            ak.b.h_n = odd ? buf.h_n1 : buf.h_n2;
            ak.b.h_m = odd ? buf.h_m1 : buf.h_m2;
            ak.b.occ = odd ? buf.occ1 : buf.occ2;
            ak.b.shadow = odd ? buf.shadow1 : buf.shadow2;
            ak.level = level;
            ak.src = SRC_QUEUE;
            ak.n_items = plan.n_samples;
            ak.n_items_dev = buf.counters + 4 * (level - 1) + 2;
            ak.b.nq_count = buf.counters + 4 * level + 2;
            // this level's hits overwrite those of level - 2, and its reflection rays the queue
            // level - 2 read: both wait for that level's shading
            if (level >= 3 && (e = cudaStreamWaitEvent(buf.aux, buf.ev_shaded[level - 2], 0)) != cudaSuccess) return e;
            ak.counter = buf.counters + 4 * level;
            if ((e = launch_march(ak, tune, buf.aux, sm_count, log, plan.spec)) != cudaSuccess) return e;
            if (level + 1 < levels && (e = launch_reflect(ak, buf.aux, log)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(buf.ev_marched[level], buf.aux)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(buf.aux2, buf.ev_marched[level], 0)) != cudaSuccess) return e;
            if (plan.ao && (e = launch_ao(ak, buf.aux2, log, plan.spec)) != cudaSuccess) return e;
            if (plan.shadows && plan.lights_max > 0) {
                ak.counter = buf.counters + 4 * level + 1;
                if ((e = launch_shadow(ak, tune, buf.aux2, sm_count, log, plan.spec)) != cudaSuccess) return e;
            }
            if ((e = launch_shade(ak, buf.aux2, log)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(buf.ev_shaded[level], buf.aux2)) != cudaSuccess) return e;
        }
        // the primary level's AO, shadows and shading overlap the reflection levels
        a0.counter = buf.counters;
        if (plan.ao && (e = launch_ao(a0, s, log, plan.spec)) != cudaSuccess) return e;
        if (plan.shadows && plan.lights_max > 0) {
            a0.counter = buf.counters + 1;
            if ((e = launch_shadow(a0, tune, s, sm_count, log, plan.spec)) != cudaSuccess) return e;
        }
        if ((e = launch_shade(a0, s, log)) != cudaSuccess) return e;
        // join: every reflection level's shading (in order on aux2) and the last march (aux)
        if ((e = cudaStreamWaitEvent(s, buf.ev_shaded[levels - 1], 0)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(s, buf.ev_marched[levels - 1], 0)) != cudaSuccess) return e;
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
    p.blur_h = buf.blur;
    return launch_post(p, s, log);
}

}  // namespace mm3e
