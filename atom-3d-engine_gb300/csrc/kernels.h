// kernels.h — host-callable launchers of the sm_103a wavefront render kernels.
//
// A beauty frame is rendered as a sequence of small kernels over ray queues (one per
// reflection level), each with a compact code footprint:
//   march   persistent tape interpreter: enhanced sphere tracing + hit normal per ray
//   ao      5-tap ambient occlusion per hit
//   shadow  persistent soft-shadow marches, one per (hit, light)
//   shade   GGX / IBL / GI / fog shading; appends reflection rays to the next level's queue
//   resolve folds the reflection levels of every AA sample and averages a pixel's samples
// followed by the post kernels (bloom, exposure, ACES, gamma, pack).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mm3e {

struct CameraArgs {
    float eye[3], fwd[3], right[3], up[3], fov_scale;
};

// Where the march kernel takes its rays from.
enum RaySource : uint32_t {
    SRC_SAMPLES = 0,  // AA camera samples: item = pixel * aa^2 + sy * aa + sx (lib.rs:1234-1240)
    SRC_CENTER = 1,   // pixel-centre camera rays (AOV / film pinhole): item = y * w + x
    SRC_QUEUE = 2,    // rays stored in the queue (reflection rays, explicit rays)
    SRC_GATHER = 3,   // GI gather rays: item = (probe * 6 + face) * dirs + d (gi.rs:75-87)
};

// Device buffers of one frame (or of one diagnostics job).
struct WaveBuffers {
    float4* q_o;         // ray origin xyz, w = sample index (uint bits)
    float4* q_d;         // ray direction xyz
    float4* h_n;         // hit normal xyz, w = t
    uint2* h_m;          // x = material id or NIL (miss), y = march steps
    float* occ;          // AO per queue slot
    float* shadow;       // per (slot * n_lights + light): < 0 light skipped, else shadow factor
    float4* nq_o;        // next level's queue
    float4* nq_d;
    uint32_t* nq_count;  // next level's queue length (device counter)
    float4* lvl;         // per sample and level: [(level * n_samples + sample) * 2 + {0, 1}]
    float4* term;        // per sample: terminal radiance xyz, w = level it ended at (uint bits)
    float4* hdr;         // per pixel output (w*h)
};

struct WaveArgs {
    const unsigned char* tape;
    uint32_t tape_bytes;
    uint32_t src;        // RaySource (march kernel)
    uint32_t level;      // reflection depth of the current queue
    uint32_t n_items;    // march: rays; shadow: rays * lights; others: rays
    const uint32_t* n_items_dev;  // if set, the item count is read from this device word
    uint32_t n_samples;  // AA samples in the frame (w * h * aa^2)
    uint32_t* counter;   // work counter for persistent kernels (zeroed per launch)
    uint32_t* status;    // error word
    CameraArgs cam;
    WaveBuffers b;
    // SRC_GATHER probe grid and direction table (6 faces x dirs_per_face, xyz + weight)
    float gi_lo[3], gi_cell[3];
    uint32_t gi_nx, gi_ny, gi_nz, dirs_per_face;
    const float4* gather_dirs;
    uint32_t aov_mode;   // RenderMode for the AOV resolve
};

// Status bits written by kernels.
enum : uint32_t { ST_TAPE_TIMEOUT = 1u, ST_TAPE_CORRUPT = 2u };

cudaError_t launch_march(const WaveArgs& a, cudaStream_t s, int sm_count, uint32_t* launches);
cudaError_t launch_ao(const WaveArgs& a, cudaStream_t s, uint32_t* launches);
cudaError_t launch_shadow(const WaveArgs& a, cudaStream_t s, int sm_count, uint32_t* launches);
cudaError_t launch_shade(const WaveArgs& a, cudaStream_t s, uint32_t* launches);
cudaError_t launch_resolve(const WaveArgs& a, uint32_t width, uint32_t height, cudaStream_t s, uint32_t* launches);
// AOV modes: display value per pixel-centre hit (lib.rs:1185-1217), written as RGBA f32.
cudaError_t launch_aov(const WaveArgs& a, uint32_t width, uint32_t height, float4* out, cudaStream_t s,
                       uint32_t* launches);
// GI gather shading: emissive + unshadowed direct light at each gather hit (lib.rs:686-711).
cudaError_t launch_gather_shade(const WaveArgs& a, float4* radiance, cudaStream_t s, uint32_t* launches);

// Post stack (post.rs:36-115): bright-pass, separable Gaussian (weights on device), add,
// exposure, ACES, gamma, clamp; output RGBA f32 or RGBA8.
struct PostArgs {
    const float4* hdr;
    float4* bright;
    float4* blur_h;
    const float* kernel_w;
    uint32_t radius;
    uint32_t width, height;
    int bloom;
    float threshold, intensity, exposure;
    int format;
    void* out;
};
cudaError_t launch_post(const PostArgs& p, cudaStream_t s, uint32_t* launches);
cudaError_t launch_pack_rgba8(const float4* src, uchar4* dst, size_t n, cudaStream_t s, uint32_t* launches);
cudaError_t launch_field(const unsigned char* tape, uint32_t tape_bytes, const float* pts, uint32_t n, float* dist,
                         uint32_t* mat, cudaStream_t s, uint32_t* launches);
cudaError_t launch_gi_reduce(const float4* radiance, const float4* dirs, uint32_t dirs_per_face, uint32_t probes,
                             float4* cubes, cudaStream_t s, uint32_t* launches);

}  // namespace mm3e
