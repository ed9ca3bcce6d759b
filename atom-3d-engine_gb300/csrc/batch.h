// batch.h — batched rendering: many scenes, cameras and resolutions in one pass sequence.
//
// Jobs are packed in order into pass sequences ("waves") whose samples fit the engine's
// capacity. A wave's job table (one FrameJob per job: tape, camera, size, sample / slot /
// pixel bases, post settings, output address) is copied to the device, and one launch per
// pass renders every job of the wave: the persistent march and shadow kernels take rays of
// all jobs from one work counter, each lane reading its own job's tape. The pass sequence is
// captured once per shape (levels, lights, AO / shadows / bloom, launch shape) as a CUDA
// graph and replayed for every wave with that shape.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <tuple>
#include <vector>

#include "capi_internal.h"

namespace mm3e {

struct WaveShape {
    uint32_t levels = 1, lights = 0;
    bool ao = false, shadows = false, bloom = false;
    uint32_t block = 128, tile_wlog = 3, unroll = 1;
    bool operator<(const WaveShape& o) const {
        return std::tie(levels, lights, ao, shadows, bloom, block, tile_wlog, unroll) <
               std::tie(o.levels, o.lights, o.ao, o.shadows, o.bloom, o.block, o.tile_wlog, o.unroll);
    }
};

// One job after validation, with its place in a wave.
struct PackedJob {
    const mm3e_job* src;
    FrameJob fj;
    size_t out_bytes;      // bytes of the frame in its format
    size_t stage_offset;   // byte offset in the host staging area (host-output jobs)
};

int status_error(mm3e_ctx* c, uint32_t status_word);

class BatchEngine {
  public:
    // `stream` null: the context's current stream.
    explicit BatchEngine(mm3e_ctx* c, cudaStream_t stream = nullptr);
    ~BatchEngine();
    int configure(const mm3e_batch_config& cfg);
    // Renders and waits; host-output jobs are copied out before it returns.
    int render(const mm3e_job* jobs, size_t n, mm3e_batch_stats* stats);
    // Enqueues the pass sequences of device-output jobs on the engine's stream and returns;
    // the caller orders later work on the stream and reads status_word() afterwards.
    int enqueue(const mm3e_job* jobs, size_t n, mm3e_batch_stats* stats);
    const uint32_t* status_word() const { return buf_.counters ? buf_.counters + (N_COUNTERS - 1) : nullptr; }
    cudaStream_t stream() const { return s_ ? s_ : c_->stream; }
    // Bytes of device memory the engine holds.
    size_t device_bytes() const;
    // Allocates the pass buffers for `samples` samples up front.
    int reserve(uint64_t samples, uint32_t lights, uint32_t levels);

  private:
    int launch_jobs(const mm3e_job* jobs, size_t n, mm3e_batch_stats& st, bool allow_host);
    int ensure(uint64_t samples, uint64_t pixels, uint32_t lights, uint32_t levels, size_t stage_bytes, uint32_t jobs,
               int ring);
    int run_wave(std::vector<PackedJob>& wave, const WaveShape& shape, uint64_t samples, uint64_t slots,
                 uint64_t pixels, mm3e_batch_stats* st, int ring);
    int flush_ring(int ring);
    cudaError_t launch_sequence(const WaveShape& shape, uint32_t* launches, bool* used_graph);

    mm3e_ctx* c_;
    cudaStream_t s_ = nullptr;
    uint64_t max_samples_ = 1ull << 24;
    bool use_graphs_ = true;
    PassBuffers buf_;
    FrameJob* d_jobs_ = nullptr;
    JobTotals* d_totals_ = nullptr;
    uint32_t job_cap_ = 0;
    // two host rings (job table + output staging), so the host fills one while the GPU works
    struct Ring {
        FrameJob* h_jobs = nullptr;
        JobTotals* h_totals = nullptr;
        unsigned char* h_stage = nullptr;  // pinned host copy of host-output frames
        unsigned char* d_stage = nullptr;  // device frames of host-output jobs
        size_t stage_cap = 0;
        cudaEvent_t done = nullptr;
        bool pending = false;
        std::vector<std::pair<void*, std::pair<size_t, size_t>>> copies;  // host dst, (offset, bytes)
    } ring_[2];
    struct GraphEntry {
        cudaGraphExec_t exec = nullptr;
        uint32_t launches = 0;
    };
    std::map<WaveShape, GraphEntry> graphs_;
    uint64_t graph_cap_ = 0;  // capacity the cached graphs were captured for
};

}  // namespace mm3e
