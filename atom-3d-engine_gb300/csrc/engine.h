// engine.h — pass sequences over frame jobs.
//
// One driver runs the beauty passes (march / AO / shadow / shade per reflection level, then
// resolve and post) for a set of frame jobs; the plain per-frame call runs it for one job
// with host-known sizes, the batched launch and the request server run it for a device job
// table with device-side sizes (so the same sequence can be captured once in a CUDA graph
// and replayed for any table that fits its buffers).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "kernels.h"

namespace mm3e {

inline uint32_t tile_w_of(uint32_t wlog) { return 1u << wlog; }
inline uint32_t tile_h_of(uint32_t wlog) { return 32u >> wlog; }
inline uint32_t tiles_x_of(uint32_t w, uint32_t wlog) { return (w + tile_w_of(wlog) - 1) / tile_w_of(wlog); }
// Pixel slots of a w x h frame in 32-pixel tiles (padding included).
inline uint64_t slots_of(uint32_t w, uint32_t h, uint32_t wlog) {
    return (uint64_t)tiles_x_of(w, wlog) * ((h + tile_h_of(wlog) - 1) / tile_h_of(wlog)) * 32u;
}

constexpr int N_COUNTERS = 64;  // [4L] march, [4L+1] shadow, [4L+2] next queue length; [63] status

constexpr int MAX_LEVELS = 8;  // bounces + 1 (MAX_BOUNCES = 7)

// Device buffers of a pass sequence: ray queues and per-sample records for `cap` samples,
// HDR / bloom arrays for `pixels` output pixels, and the work counters.
// The levels run as a pipeline: level 0 on the caller's stream; the reflection levels' marches
// (each emitting the next level's rays) in order on one auxiliary stream, forked as soon as the
// primary hits exist; and each reflection level's AO / shadows / shading on a second auxiliary
// stream as soon as its hits exist, beside the next level's march. So level 0 has queue a and hit
// set 0, and reflection level L reads queue b, c, d (rotating from L = 1) and writes hit set 1
// (odd L) or 2 (even L); a level's march waits for the shading of the level two before it, the
// last reader of the queue and hit set it overwrites.
struct PassBuffers {
    size_t cap = 0, lights = 0, levels = 0, pixels = 0;
    float4 *qa_o = nullptr, *qa_d = nullptr, *qb_o = nullptr, *qb_d = nullptr, *qc_o = nullptr, *qc_d = nullptr;
    float4 *qd_o = nullptr, *qd_d = nullptr;
    float4* h_n = nullptr;
    uint2* h_m = nullptr;
    float *occ = nullptr, *shadow = nullptr;
    float4* h_n1 = nullptr;  // hit set 1 (odd reflection levels)
    uint2* h_m1 = nullptr;
    float *occ1 = nullptr, *shadow1 = nullptr;
    float4* h_n2 = nullptr;  // hit set 2 (even reflection levels)
    uint2* h_m2 = nullptr;
    float *occ2 = nullptr, *shadow2 = nullptr;
    float4 *lvl = nullptr, *term = nullptr;
    float4 *hdr = nullptr, *blur = nullptr;
    float4* fg = nullptr;  // film coverage / foreground per output pixel
    uint32_t* counters = nullptr;
    cudaStream_t aux = nullptr;   // reflection levels' marches
    cudaStream_t aux2 = nullptr;  // reflection levels' AO / shadows / shading
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_marched[MAX_LEVELS] = {}, ev_shaded[MAX_LEVELS] = {};
    void release();
    // Grows the buffers to hold at least the given sizes (contents are not kept).
    cudaError_t ensure(size_t cap, size_t lights, size_t levels, size_t pixels);
    size_t bytes() const;
    static size_t bytes_for(size_t cap, size_t lights, size_t levels, size_t pixels);
};

// Device scratch of the G-buffer and reprojection calls: one frame of colour / depth / object
// tags, the warp's z-buffer keys, the filled mask, the hole list and the mover tables.
struct PreviewBuffers {
    size_t pixels = 0, movers = 0, deltas = 0;
    uchar4 *color = nullptr, *out = nullptr;
    float* depth = nullptr;
    int32_t* obj = nullptr;
    unsigned long long* keys = nullptr;
    unsigned char* filled = nullptr;
    uint32_t *hole_pix = nullptr, *count = nullptr;
    float4* mover = nullptr;  // centre xyz, radius
    float* delta = nullptr;   // xyz per mover
    PreviewBuffers() = default;
    PreviewBuffers(const PreviewBuffers&) = delete;
    PreviewBuffers& operator=(const PreviewBuffers&) = delete;
    ~PreviewBuffers() { release(); }
    void release();
    cudaError_t ensure(size_t pixels, size_t movers, size_t deltas);
    size_t bytes() const;
};

// Per-kernel-kind device time, from CUDA events around each pass (off by default).
class Profiler {
  public:
    ~Profiler();
    bool on = false;
    void begin(uint32_t kind, cudaStream_t s);
    void end(uint32_t kind, cudaStream_t s);
    // Waits for the recorded passes and adds their times into ms / launches; clears.
    cudaError_t collect(double* ms, uint32_t* launches);
    LaunchLog log();  // a launch log that records into this profiler when `on`

  private:
    cudaEvent_t event();
    std::vector<cudaEvent_t> pool_;
    size_t used_ = 0;
    struct Rec {
        uint32_t kind;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs_;
    std::vector<cudaEvent_t> open_;
};

// A beauty pass sequence: either one job inline (host sizes) or a device job table (sizes
// read by the kernels, buffers sized by the capacities below).
struct PassPlan {
    FrameJob job0{};
    uint32_t tape_bytes = 0;        // job0's tape (shared-memory staging)
    const FrameJob* jobs = nullptr; // device table, or null
    const JobTotals* totals = nullptr;
    uint32_t n_samples = 0;         // samples / slots / pixels (host sizes, or capacities)
    uint32_t n_slots = 0;
    uint32_t n_pixels = 0;
    uint32_t levels = 1;            // bounces + 1
    uint32_t lights_max = 0;
    bool ao = false, shadows = false, bloom = false, post = true;
    bool clear_status = true;       // also clear the status word with the work counters
    const SpecKernels* spec = nullptr;  // scene-specialised march / shadow / AO (single job only)
    bool film = false;              // resolve coverage + foreground (into buf.fg) too
    // Primary rays from queue a (count in this device word, outside buf.counters) instead of
    // the jobs' camera samples; sample k of the queue is queue entry k. The caller resolves.
    const uint32_t* queue0 = nullptr;
    uint32_t wait_limit = 0;        // tape-staging wait limit and probe mode (WaveArgs)
    uint32_t wait_probe = 0;
};

// Enqueues the passes on `s`: counters cleared, march / AO / shadow / shade per level,
// resolve into buf.hdr, then post into each job's `out` when plan.post (neither with
// plan.queue0). Asynchronous.
cudaError_t run_beauty(const PassPlan& plan, PassBuffers& buf, const TuneParams& tune, cudaStream_t s, int sm_count,
                       LaunchLog* log);

// Post stack only (hdr already in buf.hdr).
cudaError_t run_post(const PassPlan& plan, PassBuffers& buf, cudaStream_t s, int sm_count, LaunchLog* log);

}  // namespace mm3e
