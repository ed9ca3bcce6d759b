// server.cpp — the served form (continuous batching) and its C ABI.
#include "server.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>

#include "mesh.h"
#include "spec.h"

namespace mm3e {

namespace {

using Clock = std::chrono::steady_clock;

size_t round_bucket(size_t n) {
    size_t b = 64 * 1024;
    while (b < n) b <<= 1;
    return b;
}

uint64_t fnv1a(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

}  // namespace

// Device and pinned staging in power-of-two buckets (>= 64 KB), reused across requests.
class StagingPool {
  public:
    ~StagingPool() {
        for (auto& kv : dev_)
            for (void* p : kv.second) cudaFree(p);
        for (auto& kv : host_)
            for (void* p : kv.second) cudaFreeHost(p);
    }
    cudaError_t get(size_t bytes, void** d, void** h) {
        size_t b = round_bucket(bytes);
        auto& dl = dev_[b];
        auto& hl = host_[b];
        cudaError_t e = cudaSuccess;
        if (!dl.empty()) {
            *d = dl.back();
            dl.pop_back();
        } else if ((e = cudaMalloc(d, b)) != cudaSuccess) {
            return e;
        }
        if (!hl.empty()) {
            *h = hl.back();
            hl.pop_back();
        } else if ((e = cudaMallocHost(h, b)) != cudaSuccess) {
            dl.push_back(*d);
            return e;
        }
        return cudaSuccess;
    }
    void put(size_t bytes, void* d, void* h) {
        size_t b = round_bucket(bytes);
        if (d) dev_[b].push_back(d);
        if (h) host_[b].push_back(h);
    }

  private:
    std::map<size_t, std::vector<void*>> dev_, host_;
};

struct ServerScene {
    uint32_t id = 0;
    SceneCopy src;
    mm3e_scene* dev = nullptr;  // null while dropped from the device
    size_t bytes = 0;
    uint64_t last_use = 0;
    uint32_t pending = 0;       // admitted requests that render it
    bool resident = false;      // added with mm3e_server_add_scene (kept for camera updates)
    // its specialised kernels: requested from the compile workers, and the cubin once built
    // (kept on the host, so a scene dropped from the device and compiled again reloads it)
    bool spec_requested = false;
    std::shared_ptr<std::vector<char>> spec_cubin;
    uint32_t spec_block = 0;
    bool spec_smem = false;
};

// A resident scene's specialised program for the compile workers, and what they return.
struct SpecJob {
    uint32_t scene_id = 0;
    std::string source;
    uint32_t block = 0;
    bool smem = false;
};
struct SpecDone {
    uint32_t scene_id = 0;
    std::shared_ptr<std::vector<char>> cubin;
    std::string err;
    uint32_t block = 0;
    bool smem = false;
};

struct ServerRequest {
    uint64_t ticket = 0;
    mm3e_request r{};
    std::unique_ptr<SceneCopy> new_scene;
    std::vector<float> mesh_pos;
    std::vector<uint32_t> mesh_tri;
    uint32_t scene_id = 0;
    uint32_t w = 0, h = 0;
    size_t frame_bytes = 0, admit_bytes = 0;
    void *d_out = nullptr, *h_pin = nullptr;
    double t_submit = 0, t_start = 0, t_done = 0;
    int status = MM3E_OK;
    bool done = false;
};

class Server {
  public:
    Server(mm3e_ctx* ctx, const mm3e_server_config& cfg);
    ~Server();
    int init();
    int add_scene(const mm3e_scene_desc& d, uint32_t* id);
    int submit(const mm3e_request& r, uint64_t* ticket, double arrival_ms = -1.0);
    int wait(uint64_t ticket, uint32_t timeout_ms, mm3e_request_result* res);
    void stats(mm3e_server_stats* st);
    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0_).count(); }
    mm3e_ctx* ctx() { return ctx_; }

  private:
    struct Slot {
        cudaStream_t stream = nullptr;
        std::unique_ptr<BatchEngine> engine;
        PassBuffers plain_buf;           // per-frame launches: plain mode, and specialised frames
        uint32_t* h_status = nullptr;    // pinned copies of the status words (pass sequence, per-frame)
        cudaEvent_t done = nullptr;
        std::vector<ServerRequest*> reqs;
        bool busy = false;
    };
    void run();
    bool poll_slots();
    bool launch_free_slots();
    int prepare(ServerRequest* q, bool& wait_for_memory);
    int ensure_resident(ServerScene& sc, bool& wait_for_memory);
    int bake_mesh(ServerRequest* q);
    bool make_room(size_t bytes);
    void finish(ServerRequest* q, int status);
    size_t slot_bytes() const;
    void request_spec(ServerScene& sc);
    void load_spec(ServerScene& sc);
    bool poll_spec();
    void spec_worker();

    mm3e_ctx* ctx_;
    mm3e_server_config cfg_;
    Clock::time_point t0_;
    std::thread worker_;
    std::mutex mu_;
    std::condition_variable cv_in_, cv_done_;
    bool stop_ = false;
    std::deque<ServerRequest*> incoming_;                               // guarded by mu_
    std::unordered_map<uint64_t, std::unique_ptr<ServerRequest>> all_;  // guarded by mu_
    uint64_t next_ticket_ = 1;
    // worker-owned state
    std::deque<ServerRequest*> waiting_;
    std::vector<Slot> slots_;
    std::map<uint32_t, std::unique_ptr<ServerScene>> scenes_;
    uint32_t next_scene_ = 1;
    std::map<uint64_t, std::shared_ptr<std::vector<float>>> bake_cache_;
    std::map<uint64_t, mm3e_volume> bake_grid_;
    StagingPool pool_;
    uint64_t use_clock_ = 0;
    size_t admitted_ = 0;  // staging of admitted frames
    // add_scene hand-off
    struct AddJob {
        const mm3e_scene_desc* d;
        uint32_t id = 0;
        int rc = 0;
        bool done = false;
    };
    std::deque<AddJob*> adds_;  // guarded by mu_
    mm3e_server_stats st_{};    // guarded by mu_
    int init_rc_ = MM3E_OK;
    bool ready_ = false;
    // background specialisation: jobs for the compile workers and their results
    std::vector<std::thread> spec_threads_;
    std::mutex smu_;
    std::condition_variable scv_;
    std::deque<SpecJob> spec_jobs_;   // guarded by smu_
    std::deque<SpecDone> spec_done_;  // guarded by smu_
    bool spec_stop_ = false;          // guarded by smu_
};

Server::Server(mm3e_ctx* ctx, const mm3e_server_config& cfg) : ctx_(ctx), cfg_(cfg), t0_(Clock::now()) {
    if (!cfg_.hbm_budget_bytes) cfg_.hbm_budget_bytes = 40ull << 30;
    if (!cfg_.max_samples) cfg_.max_samples = 1ull << 23;
    if (!cfg_.max_inflight) cfg_.max_inflight = 2;
    cfg_.max_inflight = std::min<uint32_t>(std::max<uint32_t>(cfg_.max_inflight, 1u), 4u);
    if (cfg_.plain) cfg_.max_inflight = 1;
    if (cfg_.plain) cfg_.spec_workers = 0;
    cfg_.spec_workers = std::min<uint32_t>(cfg_.spec_workers, 64u);
    st_.budget_bytes = cfg_.hbm_budget_bytes;
}

int Server::init() {
    for (uint32_t i = 0; i < cfg_.spec_workers; ++i) spec_threads_.emplace_back([this] { spec_worker(); });
    worker_ = std::thread([this] { run(); });
    std::unique_lock<std::mutex> lk(mu_);
    cv_done_.wait(lk, [this] { return ready_; });
    return init_rc_;
}

Server::~Server() {
    {
        std::unique_lock<std::mutex> lk(mu_);
        cv_done_.wait(lk, [this] { return incoming_.empty() && st_.completed + st_.failed >= st_.submitted; });
        stop_ = true;
    }
    cv_in_.notify_all();
    if (worker_.joinable()) worker_.join();
    {
        std::lock_guard<std::mutex> lk(smu_);
        spec_stop_ = true;
        spec_jobs_.clear();
    }
    scv_.notify_all();
    for (std::thread& t : spec_threads_) t.join();
}

// ------------------------------------------------------------------------------------------
// background specialisation of resident scenes
// ------------------------------------------------------------------------------------------
// A compile worker: NVRTC-compiles queued programs (host only; no device work) until stopped.
void Server::spec_worker() {
    for (;;) {
        SpecJob job;
        {
            std::unique_lock<std::mutex> lk(smu_);
            scv_.wait(lk, [this] { return spec_stop_ || !spec_jobs_.empty(); });
            if (spec_stop_) return;
            job = std::move(spec_jobs_.front());
            spec_jobs_.pop_front();
        }
        SpecDone d;
        d.scene_id = job.scene_id;
        d.block = job.block;
        d.smem = job.smem;
        d.cubin = std::make_shared<std::vector<char>>();
        std::string err = spec_compile(job.source, *d.cubin);
        if (!err.empty() && err.compare(0, 4, "LOG:") != 0) d.err = err;
        std::lock_guard<std::mutex> lk(smu_);
        if (!spec_stop_) spec_done_.push_back(std::move(d));
    }
}

// Queue a resident scene's specialised program (worker thread; the scene is on the device).
void Server::request_spec(ServerScene& sc) {
    if (!cfg_.spec_workers || !sc.resident || sc.spec_requested || !sc.dev) return;
    sc.spec_requested = true;
    if (spec_size(sc.dev->low.blob).objects > SPEC_AUTO_MAX_OBJECTS) return;  // the interpreter is faster
    SpecJob job;
    job.scene_id = sc.id;
    const TuneParams& t = ctx_->tune;
    job.block = t.block;
    job.smem = sc.dev->low.blob.size() <= 96 * 1024;
    job.source = spec_source(sc.dev->low.blob, t.block, t.unroll, job.smem, t.min_blocks);
    {
        std::lock_guard<std::mutex> lk(smu_);
        spec_jobs_.push_back(std::move(job));
    }
    {
        std::lock_guard<std::mutex> lk(mu_);
        st_.spec_pending += 1;
    }
    scv_.notify_one();
}

// Attach a scene's built kernels to its device copy (worker thread, between launches: frames
// already queued keep the kernels they were launched with).
void Server::load_spec(ServerScene& sc) {
    if (!sc.dev || sc.dev->spec || !sc.spec_cubin) return;
    std::unique_ptr<SpecModule> m(new SpecModule());
    m->kernels.block = sc.spec_block;
    m->kernels.smem_tape = sc.spec_smem;
    if (!m->load(*sc.spec_cubin, ctx_->device).empty()) return;  // keep rendering with the interpreter
    sc.dev->spec = std::move(m);
}

// Take finished compiles and load them; true if any finished.
bool Server::poll_spec() {
    std::deque<SpecDone> done;
    {
        std::lock_guard<std::mutex> lk(smu_);
        done.swap(spec_done_);
    }
    for (SpecDone& d : done) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (st_.spec_pending) st_.spec_pending -= 1;
        }
        auto it = scenes_.find(d.scene_id);
        if (it == scenes_.end() || !d.err.empty() || d.cubin->empty()) continue;
        ServerScene& sc = *it->second;
        sc.spec_cubin = d.cubin;
        sc.spec_block = d.block;
        sc.spec_smem = d.smem;
        load_spec(sc);
        if (sc.dev && sc.dev->spec) {
            std::lock_guard<std::mutex> lk(mu_);
            st_.scenes_specialized += 1;
        }
    }
    return !done.empty();
}

size_t Server::slot_bytes() const {
    size_t b = 0;
    for (const Slot& s : slots_) b += (s.engine ? s.engine->device_bytes() : 0) + s.plain_buf.bytes();
    return b;
}

int Server::add_scene(const mm3e_scene_desc& d, uint32_t* id) {
    AddJob job;
    job.d = &d;
    {
        std::unique_lock<std::mutex> lk(mu_);
        adds_.push_back(&job);
    }
    cv_in_.notify_all();
    std::unique_lock<std::mutex> lk(mu_);
    cv_done_.wait(lk, [&] { return job.done; });
    if (job.rc == MM3E_OK && id) *id = job.id;
    return job.rc;
}

int Server::submit(const mm3e_request& r, uint64_t* ticket, double arrival_ms) {
    std::unique_ptr<ServerRequest> q(new ServerRequest());
    q->r = r;
    q->t_submit = arrival_ms >= 0.0 ? arrival_ms : now_ms();
    if (r.format != MM3E_FB_RGBA8 && r.format != MM3E_FB_RGBA_F32) return fail(ctx_, MM3E_ERR_INVALID, "unknown format");
    if (!r.host_out) return fail(ctx_, MM3E_ERR_INVALID, "null output buffer");
    if (r.new_scene) {
        std::string err;
        int rc = validate_scene(*r.new_scene, err);
        if (rc) return fail(ctx_, rc, err);
        if (r.new_scene->mode != MM3E_MODE_BEAUTY) return fail(ctx_, MM3E_ERR_UNSUPPORTED, "served scenes render beauty mode");
        q->new_scene.reset(new SceneCopy());
        q->new_scene->assign(*r.new_scene);
        if (r.mesh) {
            if (r.mesh_volume >= r.new_scene->n_volumes) return fail(ctx_, MM3E_ERR_INVALID, "mesh_volume out of range");
            q->mesh_pos.assign(r.mesh->positions, r.mesh->positions + 3 * (size_t)r.mesh->n_positions);
            q->mesh_tri.assign(r.mesh->triangles, r.mesh->triangles + 3 * (size_t)r.mesh->n_triangles);
        }
        q->r.new_scene = nullptr;
        q->r.mesh = nullptr;
    }
    std::unique_lock<std::mutex> lk(mu_);
    q->ticket = next_ticket_++;
    if (ticket) *ticket = q->ticket;
    incoming_.push_back(q.get());
    all_[q->ticket] = std::move(q);
    st_.submitted += 1;
    lk.unlock();
    cv_in_.notify_all();
    return MM3E_OK;
}

int Server::wait(uint64_t ticket, uint32_t timeout_ms, mm3e_request_result* res) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = all_.find(ticket);
    if (it == all_.end()) return fail(ctx_, MM3E_ERR_INVALID, "unknown ticket");
    ServerRequest* q = it->second.get();
    auto pred = [q] { return q->done; };
    if (timeout_ms) {
        if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return MM3E_ERR_BUSY;
    } else {
        cv_done_.wait(lk, pred);
    }
    if (res) {
        res->status = q->status;
        res->scene_id = q->scene_id;
        res->submit_ms = q->t_submit;
        res->start_ms = q->t_start;
        res->done_ms = q->t_done;
    }
    int status = q->status;
    all_.erase(it);
    return status == MM3E_OK ? MM3E_OK : status;
}

void Server::stats(mm3e_server_stats* st) {
    std::lock_guard<std::mutex> lk(mu_);
    *st = st_;
}

// ------------------------------------------------------------------------------------------
// worker
// ------------------------------------------------------------------------------------------
void Server::finish(ServerRequest* q, int status) {
    if (q->d_out || q->h_pin) pool_.put(q->frame_bytes, q->d_out, q->h_pin);
    q->d_out = q->h_pin = nullptr;
    admitted_ -= q->admit_bytes;
    q->admit_bytes = 0;
    auto it = scenes_.find(q->scene_id);
    if (it != scenes_.end() && it->second->pending > 0 && q->t_start > 0) it->second->pending -= 1;
    std::lock_guard<std::mutex> lk(mu_);
    q->status = status;
    q->t_done = now_ms();
    q->done = true;
    if (status == MM3E_OK) st_.completed += 1;
    else st_.failed += 1;
    st_.admitted_bytes = admitted_;
}

bool Server::make_room(size_t bytes) {
    // drop least-recently-used idle scenes from the device until `bytes` more fit
    for (;;) {
        size_t resident = 0;
        for (auto& kv : scenes_)
            if (kv.second->dev) resident += kv.second->bytes;
        if (resident + slot_bytes() + admitted_ + bytes <= cfg_.hbm_budget_bytes) return true;
        ServerScene* victim = nullptr;
        for (auto& kv : scenes_) {
            ServerScene* sc = kv.second.get();
            if (sc->dev && sc->pending == 0 && (!victim || sc->last_use < victim->last_use)) victim = sc;
        }
        if (!victim) return false;
        mm3e_scene_destroy(victim->dev);
        victim->dev = nullptr;
        std::lock_guard<std::mutex> lk(mu_);
        st_.scenes_evicted += 1;
    }
}

int Server::ensure_resident(ServerScene& sc, bool& wait_for_memory) {
    if (sc.dev) return MM3E_OK;
    size_t est = 0;
    if (mm3e_scene_tape_bytes(&sc.src.d, &est) != MM3E_OK) est = 0;
    for (uint32_t v = 0; v < sc.src.d.n_volumes; ++v)
        est += (size_t)sc.src.volumes[v].nx * sc.src.volumes[v].ny * sc.src.volumes[v].nz * sizeof(float);
    if (!make_room(est)) {
        wait_for_memory = true;
        return MM3E_OK;
    }
    int rc = mm3e_scene_compile(ctx_, &sc.src.d, &sc.dev);
    if (rc) return rc;
    load_spec(sc);  // a resident scene compiled again after it was dropped keeps its kernels
    sc.bytes = sc.dev->device_bytes();
    sc.last_use = ++use_clock_;
    std::lock_guard<std::mutex> lk(mu_);
    st_.scenes_compiled += 1;
    return MM3E_OK;
}

int Server::bake_mesh(ServerRequest* q) {
    const mm3e_request& r = q->r;
    uint64_t key = fnv1a(q->mesh_pos.data(), q->mesh_pos.size() * sizeof(float));
    key = fnv1a(q->mesh_tri.data(), q->mesh_tri.size() * sizeof(uint32_t), key);
    key = fnv1a(&r.mesh_resolution, sizeof(r.mesh_resolution), key);
    key = fnv1a(&r.mesh_padding, sizeof(r.mesh_padding), key);
    auto it = bake_cache_.find(key);
    std::shared_ptr<std::vector<float>> data;
    mm3e_volume grid{};
    if (it != bake_cache_.end()) {
        data = it->second;
        grid = bake_grid_[key];
        std::lock_guard<std::mutex> lk(mu_);
        st_.mesh_bake_hits += 1;
    } else {
        mm3e_mesh m{q->mesh_pos.data(), (uint32_t)(q->mesh_pos.size() / 3), q->mesh_tri.data(),
                    (uint32_t)(q->mesh_tri.size() / 3)};
        int rc = mm3e_bake_mesh_sdf(ctx_, &m, r.mesh_resolution, r.mesh_padding, &grid, nullptr, 0, 0);
        if (rc) return rc;
        data = std::make_shared<std::vector<float>>((size_t)grid.nx * grid.ny * grid.nz);
        rc = mm3e_bake_mesh_sdf(ctx_, &m, r.mesh_resolution, r.mesh_padding, &grid, data->data(), data->size(), 0);
        if (rc) return rc;
        bake_cache_[key] = data;
        bake_grid_[key] = grid;
        std::lock_guard<std::mutex> lk(mu_);
        st_.mesh_bakes += 1;
    }
    SceneCopy& sc = *q->new_scene;
    mm3e_volume& v = sc.volumes[r.mesh_volume];
    v.nx = grid.nx;
    v.ny = grid.ny;
    v.nz = grid.nz;
    std::memcpy(v.min, grid.min, 12);
    std::memcpy(v.cell, grid.cell, 12);
    sc.volume_data[r.mesh_volume] = *data;
    sc.fix();
    return MM3E_OK;
}

// Resolve a request's scene and admit its frame; sets wait_for_memory when it must wait.
int Server::prepare(ServerRequest* q, bool& wait_for_memory) {
    wait_for_memory = false;
    if (q->new_scene) {
        if (!q->mesh_pos.empty()) {
            int rc = bake_mesh(q);
            if (rc) return rc;
            q->mesh_pos.clear();
            q->mesh_tri.clear();
        }
        std::unique_ptr<ServerScene> sc(new ServerScene());
        sc->id = next_scene_++;
        sc->src.assign(q->new_scene->d);
        q->scene_id = sc->id;
        q->new_scene.reset();
        scenes_[sc->id] = std::move(sc);
    } else if (!q->scene_id) {
        q->scene_id = q->r.scene_id;
    }
    auto it = scenes_.find(q->scene_id);
    if (it == scenes_.end()) return fail(ctx_, MM3E_ERR_INVALID, "unknown scene id " + std::to_string(q->scene_id));
    ServerScene& sc = *it->second;
    int rc = ensure_resident(sc, wait_for_memory);
    if (rc || wait_for_memory) return rc;
    q->w = q->r.width ? q->r.width : sc.src.d.width;
    q->h = q->r.height ? q->r.height : sc.src.d.height;
    if (q->w == 0 || q->h == 0 || q->w > 16384 || q->h > 16384)
        return fail(ctx_, MM3E_ERR_INVALID, "dimensions must be 1..=16384");
    size_t px = q->r.format == MM3E_FB_RGBA8 ? 4 : 16;
    q->frame_bytes = (size_t)q->w * q->h * px;
    if (q->r.out_bytes < q->frame_bytes) return fail(ctx_, MM3E_ERR_INVALID, "output buffer too small");
    size_t need = round_bucket(q->frame_bytes);
    if (need + slot_bytes() > cfg_.hbm_budget_bytes)
        return fail(ctx_, MM3E_ERR_BUDGET, "frame larger than the HBM budget left beside the slot buffers");
    sc.pending += 1;  // pinned: making room for the frame must not drop the frame's own scene
    if (!make_room(need)) {
        sc.pending -= 1;
        wait_for_memory = true;
        return MM3E_OK;
    }
    cudaError_t e = pool_.get(q->frame_bytes, &q->d_out, &q->h_pin);
    if (e != cudaSuccess) {
        sc.pending -= 1;
        return cuda_fail(ctx_, e, "frame staging");
    }
    q->admit_bytes = need;
    admitted_ += need;
    sc.last_use = ++use_clock_;
    std::lock_guard<std::mutex> lk(mu_);
    st_.admitted_bytes = admitted_;
    st_.peak_admitted_bytes = std::max<uint64_t>(st_.peak_admitted_bytes, admitted_);
    return MM3E_OK;
}

bool Server::poll_slots() {
    bool any = false;
    for (Slot& s : slots_) {
        if (!s.busy) continue;
        cudaError_t e = cudaEventQuery(s.done);
        if (e == cudaErrorNotReady) continue;
        any = true;
        int status = e == cudaSuccess ? status_error(ctx_, s.h_status[0] | s.h_status[1])
                                      : cuda_fail(ctx_, e, "served pass sequence");
        for (ServerRequest* q : s.reqs) {
            if (status == MM3E_OK) std::memcpy(q->r.host_out, q->h_pin, q->frame_bytes);
            finish(q, status);
        }
        s.reqs.clear();
        s.busy = false;
        cv_done_.notify_all();
    }
    return any;
}

bool Server::launch_free_slots() {
    bool any = false;
    for (Slot& s : slots_) {
        if (s.busy || waiting_.empty()) continue;
        std::vector<ServerRequest*> batch;
        uint64_t samples = 0;
        while (!waiting_.empty()) {
            ServerRequest* q = waiting_.front();
            bool wait_mem = false;
            if (!q->d_out) {
                int rc = prepare(q, wait_mem);
                if (rc) {
                    waiting_.pop_front();
                    finish(q, rc);
                    cv_done_.notify_all();
                    any = true;
                    continue;
                }
                if (wait_mem) {
                    // arrival order: later requests wait behind it, unless nothing it could
                    // wait for is on the device or admitted (then it can never fit)
                    bool inflight = !batch.empty() || admitted_ > 0;
                    for (const Slot& o : slots_) inflight = inflight || o.busy;
                    if (!inflight) {
                        waiting_.pop_front();
                        finish(q, fail(ctx_, MM3E_ERR_BUDGET, "request does not fit the HBM budget"));
                        cv_done_.notify_all();
                        any = true;
                        continue;
                    }
                    break;
                }
            }
            const mm3e_scene* sc = scenes_[q->scene_id]->dev;
            if (!sc) {  // an admitted request's scene is pinned; never expected
                waiting_.pop_front();
                finish(q, fail(ctx_, MM3E_ERR_CUDA, "internal: admitted request lost its scene"));
                cv_done_.notify_all();
                any = true;
                continue;
            }
            uint64_t ns = slots_of(q->w, q->h, ctx_->tune.tile_wlog) * sc->low.aa * sc->low.aa;
            if (!batch.empty() && (cfg_.plain || samples + ns > cfg_.max_samples)) break;
            samples += ns;
            batch.push_back(q);
            waiting_.pop_front();
            if (cfg_.plain) break;
        }
        if (batch.empty()) break;
        any = true;
        double t = now_ms();
        for (ServerRequest* q : batch) q->t_start = t;
        int rc = MM3E_OK;
        if (cfg_.plain) {
            ServerRequest* q = batch[0];
            mm3e_scene* sc = scenes_[q->scene_id]->dev;
            PassPlan p = plain_plan(sc, q->r.camera, q->w, q->h, q->r.format, q->d_out, ctx_->tune.tile_wlog);
            cudaError_t e = s.plain_buf.ensure(p.n_samples, p.lights_max, p.levels, p.n_pixels);
            if (e == cudaSuccess) e = run_beauty(p, s.plain_buf, ctx_->tune, s.stream, ctx_->sm_count, nullptr);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s.h_status, s.plain_buf.counters + (N_COUNTERS - 1), sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, s.stream);
            if (e != cudaSuccess) rc = cuda_fail(ctx_, e, "plain frame");
            std::lock_guard<std::mutex> lk(mu_);
            st_.reserved_bytes = slot_bytes();
            st_.sequences += 1;
            st_.frames_in_sequences += 1;
        } else {
            // Requests whose scene has its specialised kernels loaded render first, each through
            // the per-frame launch sequence with those kernels (on the slot's stream and per-frame
            // buffers, sized once for the largest); the rest share one coalesced pass sequence.
            std::vector<ServerRequest*> spec_reqs, table_reqs;
            for (ServerRequest* q : batch) (scenes_[q->scene_id]->dev->spec ? spec_reqs : table_reqs).push_back(q);
            s.h_status[0] = 0;
            s.h_status[1] = 0;
            if (!spec_reqs.empty()) {
                std::vector<PassPlan> plans;
                uint64_t ns = 0, np = 0;
                uint32_t lights = 0, levels = 1;
                for (ServerRequest* q : spec_reqs) {
                    mm3e_scene* sc = scenes_[q->scene_id]->dev;
                    PassPlan p = plain_plan(sc, q->r.camera, q->w, q->h, q->r.format, q->d_out, ctx_->tune.tile_wlog);
                    p.spec = sc->spec_kernels();
                    p.clear_status = plans.empty();  // one status word for the slot's specialised frames
                    ns = std::max<uint64_t>(ns, p.n_samples);
                    np = std::max<uint64_t>(np, p.n_pixels);
                    lights = std::max(lights, p.lights_max);
                    levels = std::max(levels, p.levels);
                    plans.push_back(p);
                }
                cudaError_t e = s.plain_buf.ensure(ns, lights, levels, np);
                for (size_t i = 0; e == cudaSuccess && i < plans.size(); ++i)
                    e = run_beauty(plans[i], s.plain_buf, ctx_->tune, s.stream, ctx_->sm_count, nullptr);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(s.h_status + 1, s.plain_buf.counters + (N_COUNTERS - 1), sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, s.stream);
                if (e != cudaSuccess) rc = cuda_fail(ctx_, e, "specialised frames");
                std::lock_guard<std::mutex> lk(mu_);
                st_.sequences += spec_reqs.size();
                st_.spec_frames += spec_reqs.size();
            }
            std::vector<mm3e_job> jobs(table_reqs.size());
            for (size_t i = 0; i < table_reqs.size(); ++i) {
                ServerRequest* q = table_reqs[i];
                mm3e_job& j = jobs[i];
                j = mm3e_job{};
                j.scene = scenes_[q->scene_id]->dev;
                j.camera = q->r.camera;
                j.width = q->w;
                j.height = q->h;
                j.format = q->r.format;
                j.device_out = q->d_out;
                j.out_bytes = q->frame_bytes;
            }
            mm3e_batch_stats bst{};
            if (rc == MM3E_OK && !jobs.empty()) rc = s.engine->enqueue(jobs.data(), jobs.size(), &bst);
            if (rc == MM3E_OK && !jobs.empty()) {
                cudaError_t e = cudaMemcpyAsync(s.h_status, s.engine->status_word(), sizeof(uint32_t),
                                                cudaMemcpyDeviceToHost, s.stream);
                if (e != cudaSuccess) rc = cuda_fail(ctx_, e, "served status");
            }
            std::lock_guard<std::mutex> lk(mu_);
            st_.sequences += bst.sequences;
            st_.frames_in_sequences += batch.size();
            st_.reserved_bytes = slot_bytes();
        }
        if (rc == MM3E_OK) {
            for (ServerRequest* q : batch) {
                cudaError_t e = cudaMemcpyAsync(q->h_pin, q->d_out, q->frame_bytes, cudaMemcpyDeviceToHost, s.stream);
                if (e != cudaSuccess) {
                    rc = cuda_fail(ctx_, e, "served frame download");
                    break;
                }
            }
        }
        if (rc == MM3E_OK) {
            cudaEventRecord(s.done, s.stream);
            s.reqs = std::move(batch);
            s.busy = true;
        } else {
            cudaStreamSynchronize(s.stream);
            for (ServerRequest* q : batch) finish(q, rc);
            cv_done_.notify_all();
        }
    }
    return any;
}

void Server::run() {
    cudaSetDevice(ctx_->device);
    int rc = MM3E_OK;
    slots_.resize(cfg_.max_inflight);
    for (Slot& s : slots_) {
        cudaError_t e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&s.h_status), 2 * sizeof(uint32_t));
        if (e != cudaSuccess) {
            rc = cuda_fail(ctx_, e, "server slot");
            break;
        }
        s.h_status[0] = 0;
        s.h_status[1] = 0;
        s.engine.reset(new BatchEngine(ctx_, s.stream));
        mm3e_batch_config bc{cfg_.max_samples, cfg_.use_graphs};
        s.engine->configure(bc);
        // the slot's buffers are held for the server's life and count against the budget
        rc = cfg_.plain ? MM3E_OK : s.engine->reserve(cfg_.max_samples, 4, 2);
        if (rc) break;
    }
    {
        std::lock_guard<std::mutex> lk(mu_);
        st_.reserved_bytes = slot_bytes();
    }
    {
        std::lock_guard<std::mutex> lk(mu_);
        init_rc_ = rc;
        ready_ = true;
        if (rc) stop_ = true;
    }
    cv_done_.notify_all();
    for (;;) {
        std::vector<AddJob*> adds;
        {
            std::unique_lock<std::mutex> lk(mu_);
            bool idle = waiting_.empty();
            for (const Slot& s : slots_) idle = idle && !s.busy;
            if (idle && incoming_.empty() && adds_.empty()) {
                if (stop_) break;
                cv_in_.wait_for(lk, std::chrono::milliseconds(2));
            }
            while (!incoming_.empty()) {
                waiting_.push_back(incoming_.front());
                incoming_.pop_front();
            }
            adds.assign(adds_.begin(), adds_.end());
            adds_.clear();
        }
        for (AddJob* a : adds) {
            std::string err;
            int arc = validate_scene(*a->d, err);
            if (arc) fail(ctx_, arc, err);
            else if (a->d->mode != MM3E_MODE_BEAUTY) arc = fail(ctx_, MM3E_ERR_UNSUPPORTED, "served scenes render beauty mode");
            uint32_t id = 0;
            if (!arc) {
                std::unique_ptr<ServerScene> sc(new ServerScene());
                sc->id = next_scene_++;
                sc->src.assign(*a->d);
                sc->resident = true;
                bool wait_mem = false;
                arc = ensure_resident(*sc, wait_mem);
                if (!arc) {
                    request_spec(*sc);
                    id = sc->id;
                    scenes_[sc->id] = std::move(sc);
                }
            }
            std::lock_guard<std::mutex> lk(mu_);
            a->rc = arc;
            a->id = id;
            a->done = true;
            cv_done_.notify_all();
        }
        bool progressed = poll_spec();
        progressed = poll_slots() || progressed;
        progressed = launch_free_slots() || progressed;
        if (!progressed) {
            bool busy = false;
            for (const Slot& s : slots_) busy = busy || s.busy;
            if (busy) std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
    }
    for (Slot& s : slots_) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        s.engine.reset();
        s.plain_buf.release();
        if (s.h_status) cudaFreeHost(s.h_status);
        if (s.done) cudaEventDestroy(s.done);
        if (s.stream) cudaStreamDestroy(s.stream);
    }
    for (auto& kv : scenes_)
        if (kv.second->dev) mm3e_scene_destroy(kv.second->dev);
    scenes_.clear();
}

}  // namespace mm3e

using namespace mm3e;

extern "C" {

int mm3e_server_create(mm3e_ctx* ctx, const mm3e_server_config* cfg, mm3e_server** out) {
    if (!ctx || !out) return MM3E_ERR_INVALID;
    *out = nullptr;
    mm3e_server_config c = cfg ? *cfg : mm3e_server_config{};
    std::unique_ptr<mm3e_server> s(new mm3e_server());
    s->impl.reset(new Server(ctx, c));
    int rc = s->impl->init();
    if (rc) return rc;
    *out = s.release();
    return MM3E_OK;
}

int mm3e_server_add_scene(mm3e_server* srv, const mm3e_scene_desc* desc, uint32_t* scene_id) {
    if (!srv || !desc) return MM3E_ERR_INVALID;
    return srv->impl->add_scene(*desc, scene_id);
}

int mm3e_server_submit(mm3e_server* srv, const mm3e_request* req, uint64_t* ticket) {
    if (!srv || !req) return MM3E_ERR_INVALID;
    return srv->impl->submit(*req, ticket);
}

int mm3e_server_wait(mm3e_server* srv, uint64_t ticket, uint32_t timeout_ms, mm3e_request_result* result) {
    if (!srv) return MM3E_ERR_INVALID;
    return srv->impl->wait(ticket, timeout_ms, result);
}

int mm3e_server_get_stats(mm3e_server* srv, mm3e_server_stats* stats) {
    if (!srv || !stats) return MM3E_ERR_INVALID;
    srv->impl->stats(stats);
    return MM3E_OK;
}

int mm3e_server_replay(mm3e_server* srv, const mm3e_request* reqs, const double* arrival_s, size_t n,
                       mm3e_request_result* results) {
    if (!srv || (n && (!reqs || !arrival_s || !results))) return MM3E_ERR_INVALID;
    Server& s = *srv->impl;
    std::vector<uint64_t> tickets(n, 0);
    std::vector<int> submit_rc(n, MM3E_OK);
    double base = s.now_ms();
    auto t_base = std::chrono::steady_clock::now();
    std::thread driver([&] {
        for (size_t i = 0; i < n; ++i) {
            auto due = t_base + std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                                    std::chrono::duration<double>(arrival_s[i]));
            auto now = std::chrono::steady_clock::now();
            if (due > now + std::chrono::microseconds(200))
                std::this_thread::sleep_until(due - std::chrono::microseconds(100));
            while (std::chrono::steady_clock::now() < due) {
            }
            submit_rc[i] = s.submit(reqs[i], &tickets[i], base + arrival_s[i] * 1000.0);
        }
    });
    driver.join();
    int rc = MM3E_OK;
    for (size_t i = 0; i < n; ++i) {
        mm3e_request_result& r = results[i];
        r = mm3e_request_result{};
        if (submit_rc[i]) {
            r.status = submit_rc[i];
            rc = submit_rc[i];
            continue;
        }
        s.wait(tickets[i], 0, &r);
        r.submit_ms -= base;
        r.start_ms -= base;
        r.done_ms -= base;
        if (r.status) rc = r.status;
    }
    return rc;
}

void mm3e_server_destroy(mm3e_server* srv) { delete srv; }

}  // extern "C"
