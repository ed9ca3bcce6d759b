// batch.cpp — BatchEngine (batched pass sequences) and its C ABI, plus the autotuner.
#include "batch.h"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace mm3e {

int status_error(mm3e_ctx* c, uint32_t st);

namespace {
constexpr uint32_t WAVE_JOBS_MAX = 4096;

int check_wave_status(mm3e_ctx* c, cudaStream_t s, const uint32_t* d_status) {
    uint32_t st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch render");
    return status_error(c, st);
}
}  // namespace

int status_error(mm3e_ctx* c, uint32_t st) {
    if (st & ST_TAPE_TIMEOUT) return fail(c, MM3E_ERR_TIMEOUT, "scene tape staging wait gave up");
    if (st & ST_TAPE_CORRUPT) return fail(c, MM3E_ERR_CUDA, "scene tape corrupt after staging");
    return MM3E_OK;
}

BatchEngine::BatchEngine(mm3e_ctx* c, cudaStream_t stream) : c_(c), s_(stream) {
    for (Ring& r : ring_) cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming);
}

BatchEngine::~BatchEngine() {
    cudaSetDevice(c_->device);
    cudaStreamSynchronize(stream());
    for (auto& g : graphs_) cudaGraphExecDestroy(g.second.exec);
    buf_.release();
    cudaFree(d_jobs_);
    cudaFree(d_totals_);
    for (Ring& r : ring_) {
        cudaFreeHost(r.h_jobs);
        cudaFreeHost(r.h_totals);
        cudaFreeHost(r.h_stage);
        cudaFree(r.d_stage);
        cudaEventDestroy(r.done);
    }
}

size_t BatchEngine::device_bytes() const {
    size_t b = buf_.bytes() + (size_t)job_cap_ * sizeof(FrameJob);
    for (const Ring& r : ring_) b += r.stage_cap;
    return b;
}

int BatchEngine::reserve(uint64_t samples, uint32_t lights, uint32_t levels) {
    cudaError_t e = buf_.ensure(samples, lights, levels, samples);
    return e == cudaSuccess ? MM3E_OK : cuda_fail(c_, e, "batch buffer allocation");
}

int BatchEngine::configure(const mm3e_batch_config& cfg) {
    uint64_t cap = cfg.max_samples ? cfg.max_samples : (1ull << 24);
    if (cap > 0x7FFFFFFFull) return fail(c_, MM3E_ERR_INVALID, "max_samples too large");
    cudaError_t e = cudaStreamSynchronize(stream());
    if (e != cudaSuccess) return cuda_fail(c_, e, "batch configure");
    max_samples_ = cap;
    use_graphs_ = cfg.use_graphs != 0;
    return MM3E_OK;
}

int BatchEngine::ensure(uint64_t samples, uint64_t pixels, uint32_t lights, uint32_t levels, size_t stage_bytes,
                        uint32_t jobs, int ring) {
    bool regrow = samples > buf_.cap || pixels > buf_.pixels || lights > buf_.lights || levels > buf_.levels;
    if (regrow) {
        cudaStreamSynchronize(stream());
        for (auto& g : graphs_) cudaGraphExecDestroy(g.second.exec);
        graphs_.clear();
        // grow geometrically up to the configured capacity (the captured graphs are redone)
        uint64_t cap = std::max<uint64_t>(samples, std::min<uint64_t>(max_samples_, 2 * (uint64_t)buf_.cap));
        cap = std::max<uint64_t>(cap, pixels);
        cudaError_t e = buf_.ensure(cap, std::max<size_t>(lights, buf_.lights), std::max<size_t>(levels, buf_.levels), cap);
        if (e != cudaSuccess) return cuda_fail(c_, e, "batch buffer allocation");
    }
    if (jobs > job_cap_) {
        cudaStreamSynchronize(stream());
        cudaFree(d_jobs_);
        cudaFree(d_totals_);
        d_jobs_ = nullptr;
        d_totals_ = nullptr;
        for (Ring& r : ring_) {
            cudaFreeHost(r.h_jobs);
            cudaFreeHost(r.h_totals);
            r.h_jobs = nullptr;
            r.h_totals = nullptr;
        }
        for (auto& g : graphs_) cudaGraphExecDestroy(g.second.exec);
        graphs_.clear();
        uint32_t cap = std::max<uint32_t>(jobs, 256u);
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d_jobs_), cap * sizeof(FrameJob));
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_totals_), sizeof(JobTotals));
        for (Ring& r : ring_) {
            if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r.h_jobs), cap * sizeof(FrameJob));
            if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r.h_totals), sizeof(JobTotals));
        }
        if (e != cudaSuccess) {
            job_cap_ = 0;
            return cuda_fail(c_, e, "batch job table allocation");
        }
        job_cap_ = cap;
    }
    {
        Ring& r = ring_[ring];  // the other ring may still hold frames to copy out
        if (stage_bytes > r.stage_cap) {
            cudaStreamSynchronize(stream());
            cudaFreeHost(r.h_stage);
            cudaFree(r.d_stage);
            r.h_stage = nullptr;
            r.d_stage = nullptr;
            r.stage_cap = 0;
            cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&r.h_stage), stage_bytes);
            if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&r.d_stage), stage_bytes);
            if (e != cudaSuccess) return cuda_fail(c_, e, "batch staging allocation");
            r.stage_cap = stage_bytes;
        }
    }
    return MM3E_OK;
}

// Enqueue the pass sequence for the device table (captured as a graph per shape).
cudaError_t BatchEngine::launch_sequence(const WaveShape& shape, uint32_t* launches, bool* used_graph) {
    PassPlan p;
    p.clear_status = false;  // one status word for all waves of a call
    p.jobs = d_jobs_;
    p.totals = d_totals_;
    p.n_samples = (uint32_t)buf_.cap;
    p.n_slots = (uint32_t)buf_.cap;
    p.n_pixels = (uint32_t)buf_.pixels;
    p.levels = shape.levels;
    p.lights_max = shape.lights;
    p.ao = shape.ao;
    p.shadows = shape.shadows;
    p.bloom = shape.bloom;
    TuneParams t;
    t.block = shape.block;
    t.tile_wlog = shape.tile_wlog;
    t.unroll = shape.unroll;
    *used_graph = false;
    if (!use_graphs_ || c_->prof.on) {
        LaunchLog log = c_->prof.log();
        cudaError_t e = run_beauty(p, buf_, t, stream(), c_->sm_count, &log);
        *launches += log.launches;
        return e;
    }
    auto it = graphs_.find(shape);
    if (it == graphs_.end()) {
        cudaStream_t cs = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
        LaunchLog log;
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        cudaError_t e2 = cudaSuccess;
        if (e == cudaSuccess) {
            e2 = run_beauty(p, buf_, t, cs, c_->sm_count, &log);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(cs, &g);
            GraphEntry ge;
            ge.launches = log.launches;
            if (e == cudaSuccess && e2 == cudaSuccess) e = cudaGraphInstantiate(&ge.exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e == cudaSuccess && e2 == cudaSuccess) it = graphs_.emplace(shape, ge).first;
        }
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) return e;
        if (e2 != cudaSuccess) return e2;
    }
    *launches += it->second.launches;
    *used_graph = true;
    return cudaGraphLaunch(it->second.exec, stream());
}

// Copy the host-output frames of a finished ring to their caller buffers.
int BatchEngine::flush_ring(int ring) {
    Ring& r = ring_[ring];
    if (!r.pending) return MM3E_OK;
    cudaError_t e = cudaEventSynchronize(r.done);
    if (e != cudaSuccess) return cuda_fail(c_, e, "batch output");
    for (auto& cp : r.copies) std::memcpy(cp.first, r.h_stage + cp.second.first, cp.second.second);
    r.copies.clear();
    r.pending = false;
    return MM3E_OK;
}

int BatchEngine::run_wave(std::vector<PackedJob>& wave, const WaveShape& shape, uint64_t samples, uint64_t slots,
                          uint64_t pixels, mm3e_batch_stats* st, int ring) {
    int rc = flush_ring(ring);  // the ring's host buffers are reused below
    if (rc) return rc;
    Ring& r = ring_[ring];
    size_t stage = 0;
    for (const PackedJob& pj : wave)
        if (!pj.src->device_out) stage += (pj.out_bytes + 255) & ~(size_t)255;
    rc = ensure(samples, pixels, shape.lights, shape.levels, stage, (uint32_t)wave.size(), ring);
    if (rc) return rc;
    for (size_t i = 0; i < wave.size(); ++i) {
        PackedJob& pj = wave[i];
        if (!pj.src->device_out) pj.fj.out = r.d_stage + pj.stage_offset;
        r.h_jobs[i] = pj.fj;
    }
    *r.h_totals = JobTotals{(uint32_t)wave.size(), (uint32_t)samples, (uint32_t)slots, (uint32_t)pixels};
    cudaStream_t s = stream();
    cudaError_t e = cudaMemcpyAsync(d_jobs_, r.h_jobs, wave.size() * sizeof(FrameJob), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_totals_, r.h_totals, sizeof(JobTotals), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(c_, e, "batch job table upload");
    uint32_t launches = 0;
    bool graph = false;
    e = launch_sequence(shape, &launches, &graph);
    if (e != cudaSuccess) return cuda_fail(c_, e, "batch pass sequence");
    uint64_t d2h = 0;
    for (const PackedJob& pj : wave) {
        if (pj.src->device_out) continue;
        e = cudaMemcpyAsync(r.h_stage + pj.stage_offset, r.d_stage + pj.stage_offset, pj.out_bytes,
                            cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_fail(c_, e, "batch output download");
        r.copies.push_back({pj.src->host_out, {pj.stage_offset, pj.out_bytes}});
        d2h += pj.out_bytes;
    }
    e = cudaEventRecord(r.done, s);
    if (e != cudaSuccess) return cuda_fail(c_, e, "batch event");
    r.pending = true;
    if (st) {
        st->sequences += 1;
        st->kernel_launches += launches;
        st->graph_launches += graph ? 1u : 0u;
        st->samples += samples;
        st->h2d_bytes += wave.size() * sizeof(FrameJob) + sizeof(JobTotals);
        st->d2h_bytes += d2h;
    }
    return MM3E_OK;
}

int BatchEngine::launch_jobs(const mm3e_job* jobs, size_t n, mm3e_batch_stats& st, bool allow_host) {
    if (n && !jobs) return fail(c_, MM3E_ERR_INVALID, "null job array");
    const uint32_t wlog = c_->tune.tile_wlog;
    // validate and size every job first
    std::vector<PackedJob> packed(n);
    uint64_t largest = 0;
    for (size_t i = 0; i < n; ++i) {
        const mm3e_job& j = jobs[i];
        if (!j.scene || j.scene->ctx != c_ || !c_->scenes.count(j.scene))
            return fail(c_, MM3E_ERR_INVALID, "job " + std::to_string(i) + ": not a scene of this context");
        const mm3e_scene* s = j.scene;
        if (s->low.mode != MM3E_MODE_BEAUTY)
            return fail(c_, MM3E_ERR_UNSUPPORTED, "job " + std::to_string(i) + ": batched jobs render beauty mode");
        if (j.format != MM3E_FB_RGBA8 && j.format != MM3E_FB_RGBA_F32)
            return fail(c_, MM3E_ERR_INVALID, "job " + std::to_string(i) + ": unknown framebuffer format");
        uint32_t w = j.width ? j.width : s->low.width, h = j.height ? j.height : s->low.height;
        if (w == 0 || h == 0 || w > 16384 || h > 16384)
            return fail(c_, MM3E_ERR_INVALID, "job " + std::to_string(i) + ": dimensions must be 1..=16384");
        size_t px = j.format == MM3E_FB_RGBA8 ? 4 : 16;
        size_t bytes = (size_t)w * h * px;
        void* out = j.device_out ? j.device_out : (allow_host ? j.host_out : nullptr);
        if (!out || j.out_bytes < bytes)
            return fail(c_, MM3E_ERR_INVALID, "job " + std::to_string(i) + ": output buffer too small");
        PackedJob& pj = packed[i];
        pj.src = &j;
        pj.fj = scene_job(s, nullptr, j.camera, w, h, wlog);
        pj.fj.format = j.format;
        pj.fj.out = j.device_out;
        pj.out_bytes = bytes;
        largest = std::max<uint64_t>(largest, pj.fj.n_samples);
    }
    if (largest > 0x7FFFFFFFull) return fail(c_, MM3E_ERR_INVALID, "job too large");
    uint64_t cap = std::max<uint64_t>(max_samples_, largest);
    cudaSetDevice(c_->device);
    std::vector<PackedJob> wave;
    WaveShape shape;
    uint64_t samples = 0, slots = 0, pixels = 0;
    size_t stage = 0;
    int ring = 0;
    if (buf_.counters) {  // status word of the previous call
        cudaError_t e = cudaMemsetAsync(buf_.counters + (N_COUNTERS - 1), 0, sizeof(uint32_t), stream());
        if (e != cudaSuccess) return cuda_fail(c_, e, "batch status");
    }
    auto emit = [&]() -> int {
        if (wave.empty()) return MM3E_OK;
        shape.block = c_->tune.block;
        shape.tile_wlog = wlog;
        shape.unroll = c_->tune.unroll;
        int rc = run_wave(wave, shape, samples, slots, pixels, &st, ring);
        ring ^= 1;
        wave.clear();
        shape = WaveShape();
        samples = slots = pixels = 0;
        stage = 0;
        return rc;
    };
    for (size_t i = 0; i < n; ++i) {
        PackedJob pj = packed[i];
        if (!wave.empty() && (samples + pj.fj.n_samples > cap || wave.size() >= WAVE_JOBS_MAX)) {
            int rc = emit();
            if (rc) return rc;
        }
        const mm3e_scene* s = pj.src->scene;
        const TapeHeader* h = reinterpret_cast<const TapeHeader*>(s->low.blob.data());
        pj.fj.sample_base = (uint32_t)samples;
        pj.fj.slot_base = (uint32_t)slots;
        pj.fj.pixel_base = (uint32_t)pixels;
        pj.stage_offset = stage;
        if (!pj.src->device_out) stage += (pj.out_bytes + 255) & ~(size_t)255;
        samples += pj.fj.n_samples;
        slots += pj.fj.n_slots;
        pixels += pj.fj.n_pixels;
        shape.levels = std::max(shape.levels, s->low.bounces + 1);
        shape.lights = std::max(shape.lights, h->n_lights);
        shape.ao = shape.ao || ((h->flags & SF_AO) && h->ao_samples > 0);
        shape.shadows = shape.shadows || ((h->flags & SF_SHADOWS) && h->shadow_steps > 0 && h->n_lights > 0);
        shape.bloom = shape.bloom || (pj.fj.flags & JF_BLOOM);
        wave.push_back(pj);
    }
    return emit();
}

int BatchEngine::render(const mm3e_job* jobs, size_t n, mm3e_batch_stats* stats) {
    auto t0 = std::chrono::steady_clock::now();
    mm3e_batch_stats st{};
    cudaSetDevice(c_->device);
    cudaEventRecord(c_->ev0, stream());
    int rc = launch_jobs(jobs, n, st, true);
    if (rc) return rc;
    cudaEventRecord(c_->ev1, stream());
    rc = check_wave_status(c_, stream(), buf_.counters + (N_COUNTERS - 1));
    if (rc) return rc;
    for (int r = 0; r < 2; ++r) {
        rc = flush_ring(r);
        if (rc) return rc;
    }
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, c_->ev0, c_->ev1);
        st.device_ms = ms;
        st.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        *stats = st;
    }
    return MM3E_OK;
}

int BatchEngine::enqueue(const mm3e_job* jobs, size_t n, mm3e_batch_stats* stats) {
    mm3e_batch_stats st{};
    int rc = launch_jobs(jobs, n, st, false);
    if (stats) *stats = st;
    return rc;
}


}  // namespace mm3e

using namespace mm3e;

extern "C" {

int mm3e_batch_configure(mm3e_ctx* ctx, const mm3e_batch_config* cfg) {
    if (!ctx || !cfg) return MM3E_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (!ctx->batch) ctx->batch.reset(new BatchEngine(ctx));
    return ctx->batch->configure(*cfg);
}

int mm3e_render_batch(mm3e_ctx* ctx, const mm3e_job* jobs, size_t n, mm3e_batch_stats* stats) {
    if (!ctx) return MM3E_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (!ctx->batch) ctx->batch.reset(new BatchEngine(ctx));
    return ctx->batch->render(jobs, n, stats);
}

int mm3e_autotune(mm3e_ctx* ctx, const mm3e_job* jobs, size_t n, uint32_t repeats, mm3e_tuning* best,
                  mm3e_tune_entry* report, uint32_t report_cap, uint32_t* n_report) {
    if (!ctx || (n && !jobs)) return MM3E_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (!ctx->batch) ctx->batch.reset(new BatchEngine(ctx));
    TuneParams keep = ctx->tune;
    const uint32_t blocks[2] = {128, 256}, wlogs[3] = {2, 3, 4}, unrolls[3] = {1, 16, 64};
    double best_ms = -1.0;
    TuneParams best_t = keep;
    uint32_t k = 0;
    for (uint32_t b : blocks)
        for (uint32_t wl : wlogs)
            for (uint32_t u : unrolls) {
                ctx->tune.block = b;
                ctx->tune.tile_wlog = wl;
                ctx->tune.unroll = u;
                mm3e_batch_stats st{};
                int rc = ctx->batch->render(jobs, n, &st);  // warm-up (captures the graphs)
                double ms = 0.0;
                for (uint32_t r = 0; rc == MM3E_OK && r < (repeats ? repeats : 1); ++r) {
                    rc = ctx->batch->render(jobs, n, &st);
                    ms += st.device_ms;
                }
                if (rc) {
                    ctx->tune = keep;
                    return rc;
                }
                ms /= (repeats ? repeats : 1);
                if (report && k < report_cap) {
                    report[k].tuning.block = b;
                    report[k].tuning.tile_wlog = wl;
                    report[k].tuning.unroll = u;
                    report[k].tuning.min_blocks = keep.min_blocks;
                    report[k].device_ms = ms;
                }
                ++k;
                if (best_ms < 0.0 || ms < best_ms) {
                    best_ms = ms;
                    best_t = ctx->tune;
                }
            }
    ctx->tune = best_t;
    if (best) {
        best->block = best_t.block;
        best->tile_wlog = best_t.tile_wlog;
        best->unroll = best_t.unroll;
        best->min_blocks = best_t.min_blocks;
    }
    if (n_report) *n_report = k;
    return MM3E_OK;
}

}  // extern "C"
