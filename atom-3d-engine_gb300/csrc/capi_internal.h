// capi_internal.h — the C ABI's opaque handles and the helpers the ABI files share.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <set>
#include <string>
#include <vector>

#include "../../include/mm3e_cuda.h"
#include "engine.h"
#include "kernels.h"
#include "lower.h"

namespace mm3e {
class BatchEngine;
class SpecModule;
}

struct mm3e_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;      // stream all work is issued on
    cudaStream_t own_stream = nullptr;  // the context's own stream
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int sm_count = 0, clock_khz = 0;
    // The device reaches pageable host memory through the host's page tables (a coherent
    // NVLink-C2C host such as Grace): kernels then write host framebuffers directly.
    bool host_access = false;
    bool host_writes = true;  // use that for host outputs (mm3e_ctx_set_host_writes)
    uint32_t wait_limit = 0;  // tape-staging wait limit of the plain calls (mm3e_ctx_set_tape_wait)
    uint32_t wait_probe = 0;
    std::string err;
    std::set<mm3e_scene*> scenes;       // live scenes; destroyed with the context
    mm3e::TuneParams tune;              // launch shape of the march / shadow passes
    mm3e::Profiler prof;                // per-kernel device time (off by default)
    double kk_ms[mm3e::KK_COUNT] = {};
    uint32_t kk_launches[mm3e::KK_COUNT] = {};
    std::unique_ptr<mm3e::BatchEngine> batch;
    mm3e::PreviewBuffers preview;       // render_gbuffer / reproject scratch
    ~mm3e_ctx();
};

namespace mm3e {

// Owned deep copy of a scene description (host), so dynamic spheres and GI bakes can
// re-lower the scene after the caller has released its arrays.
struct SceneCopy {
    mm3e_scene_desc d{};
    std::vector<mm3e_object> objects;
    std::vector<mm3e_material> materials;
    std::vector<mm3e_light> lights;
    std::vector<mm3e_volume> volumes;
    std::vector<std::vector<float>> volume_data;
    std::vector<mm3e_csg_node> csg_nodes;
    std::vector<uint32_t> csg_roots;
    bool has_gi = false;
    mm3e_gi gi{};
    std::vector<float> gi_cubes;
    void assign(const mm3e_scene_desc& s);
    void fix();
};

int fail(mm3e_ctx* c, int code, const std::string& msg);
int cuda_fail(mm3e_ctx* c, cudaError_t e, const char* what);
void fill_camera(CameraArgs& a, const mm3e_camera& c);

}  // namespace mm3e

struct mm3e_scene {
    mm3e_ctx* ctx = nullptr;
    mm3e::SceneCopy src;
    mm3e::LoweredScene low;
    unsigned char* d_tape = nullptr;
    size_t tape_cap = 0;
    unsigned char* d_dyn_tape = nullptr;  // tape with dynamic spheres appended
    size_t dyn_cap = 0;
    std::vector<void*> d_payloads;        // same order as low.payloads
    float* d_kernel = nullptr;            // bloom weights
    uint32_t bloom_radius = 0;
    float4* d_out = nullptr;              // framebuffer for host copies (w*h float4)
    void* h_stage = nullptr;              // pinned staging (w*h*16 bytes)
    size_t pixels = 0;
    mm3e::PassBuffers buf;                // frame ray queues, hit records, HDR / bloom, counters
    uint32_t buf_wlog = 3;                // tile shape the buffers were sized for
    std::unique_ptr<mm3e::SpecModule> spec;  // scene-specialised kernels (NVRTC), when built
    mm3e::TuneParams tune;                // this scene's launch shape (mm3e_scene_autotune) ...
    bool own_tune = false;                // ... used instead of the context's when set
    const mm3e::TuneParams& tuning() const { return own_tune ? tune : ctx->tune; }
    const mm3e::SpecKernels* spec_kernels() const;
    ~mm3e_scene();
    uint32_t n_lights() const;
    size_t device_bytes() const;          // tape + payloads + frame buffers
};

namespace mm3e {
// A frame job of `s` (its tape, or `tape` when given) for `cam` at w x h (0: the scene's).
FrameJob scene_job(const mm3e_scene* s, const unsigned char* tape, const mm3e_camera& cam, uint32_t w, uint32_t h,
                   uint32_t wlog);
// The per-frame launch sequence's plan (one inline job, tape staged in shared memory) for a
// beauty frame of `s` at w x h (0: the scene's) into device memory `dout`.
PassPlan plain_plan(const mm3e_scene* s, const mm3e_camera& cam, uint32_t w, uint32_t h, uint32_t format, void* dout,
                    uint32_t wlog);
}  // namespace mm3e
