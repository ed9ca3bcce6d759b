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
//
// Every pass works on a set of frame jobs (scene tape + camera + resolution + output): the
// plain per-frame call is a set of one job passed inline in the kernel parameters; the
// batched and served forms put many jobs of different scenes and sizes into one pass
// sequence through a device-resident job table, so one launch per pass covers all of them.
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#include <stdint.h>
#endif

namespace mm3e {

struct CameraArgs {
    float eye[3], fwd[3], right[3], up[3], fov_scale;
};

// Where the march kernel takes its rays from.
enum RaySource : uint32_t {
    SRC_SAMPLES = 0,  // AA camera samples of the jobs: item = job.sample_base + slot * spp + sub
    SRC_CENTER = 1,   // pixel-centre camera rays of job 0 (AOV / film pinhole): item = y * w + x
    SRC_QUEUE = 2,    // rays stored in the queue (reflection rays, explicit rays)
    SRC_GATHER = 3,   // GI gather rays of job 0: item = (probe * 6 + face) * dirs + d (gi.rs:75-87)
};

// Job flags
enum : uint32_t { JF_BLOOM = 1u };

// One frame of a pass sequence. Sample slots: the job's pixels in tiles of 32 (tile shape
// from the launch), padding included, times aa^2 samples, starting at sample_base; pixel
// slots (padded) start at slot_base; output pixels (row-major) start at pixel_base of the
// pass sequence's HDR / bloom arrays.
struct FrameJob {
    const unsigned char* tape;  // device scene tape
    const float* bloom_w;       // 2r+1 normalised Gaussian weights (device)
    void* out;                  // device output, width*height RGBA8 or RGBA f32 (post only)
    CameraArgs cam;
    uint32_t width, height, aa, spp;
    uint32_t tiles_x;           // tiles per row
    uint32_t sample_base, n_samples;
    uint32_t slot_base, n_slots;
    uint32_t pixel_base, n_pixels;
    uint32_t n_lights;
    uint32_t bloom_radius, format, flags;
    float threshold, intensity, exposure;
    float lens_radius, focus_distance;  // thin lens (camera.rs Lens); radius 0: pinhole
};

// Sizes of a device job table (read by the kernels when the table is on the device).
struct JobTotals {
    uint32_t n_jobs, n_samples, n_slots, n_pixels;
};

// Launch shape of the march / shadow passes (the autotuner's search space).
struct TuneParams {
    uint32_t block = 128;    // threads per CTA: 128 or 256
    uint32_t tile_wlog = 3;  // pixel tile 2^tile_wlog x 2^(5 - tile_wlog): 8x4 by default
    uint32_t unroll = 64;    // field samples per lane between refills (the interpreter: 1, 16 or 64)
    uint32_t min_blocks = 0; // specialised kernels: CTAs per SM the register budget must allow (0: free)
};

// Device buffers of one pass sequence.
struct WaveBuffers {
    float4* q_o;         // ray origin xyz, w = sample slot (uint bits)
    float4* q_d;         // ray direction xyz, w = job index (uint bits)
    float4* h_n;         // hit normal xyz, w = t
    uint2* h_m;          // x = material id or NIL (miss), y = march steps
    float* occ;          // AO per queue slot
    float* shadow;       // per (slot * lights_max + light): < 0 light skipped, else shadow factor
    float4* nq_o;        // next level's queue
    float4* nq_d;
    uint32_t* nq_count;  // next level's queue length (device counter)
    float4* lvl;         // per sample and level: [(level * cap + sample) * 2 + {0, 1}]
    float4* term;        // per sample: terminal radiance xyz, w = level it ended at (uint bits)
    float4* hdr;         // per output pixel (job.pixel_base + y * w + x)
    float4* fg;          // film: premultiplied foreground per output pixel
};

struct WaveArgs {
    FrameJob job0;              // the job when `jobs` is null
    const FrameJob* jobs;       // device job table, or null
    const JobTotals* totals;    // device sizes of the table (with `jobs`)
    uint32_t n_jobs;            // with job0: 1
    uint32_t tape_bytes;        // bytes of job0's tape (shared-memory staging)
    uint32_t src;               // RaySource (march kernel)
    uint32_t level;             // reflection depth of the current queue
    uint32_t n_items;           // items of the pass when known on the host (else its capacity)
    const uint32_t* n_items_dev;  // if set, the item count is read from this device word
    uint32_t cap;               // sample capacity of the buffers (level stride of `lvl`)
    uint32_t lights_max;        // shadow items per queue slot
    uint32_t tile_wlog;
    uint32_t grid_cap;          // block limit of the grid-stride kernels (0: one thread per item)
    uint32_t* counter;          // work counter for persistent kernels (zeroed per launch)
    uint32_t* status;           // error word
    WaveBuffers b;
    // SRC_GATHER probe grid and direction table (6 faces x dirs_per_face, xyz + weight)
    float gi_lo[3], gi_cell[3];
    uint32_t gi_nx, gi_ny, gi_nz, dirs_per_face;
    const float4* gather_dirs;
    uint32_t aov_mode;          // RenderMode for the AOV resolve
    uint32_t emit;              // shade appends reflection rays (else a reflect pass did)
    uint32_t film;              // resolve also writes coverage (hdr.w) and the foreground (b.fg)
    uint32_t wait_limit;        // iterations of the tape-staging wait before it gives up (0: 2^22)
    uint32_t wait_probe;        // 1: issue no tape copy, so the staging wait runs to its limit
};

// Status bits written by kernels.
enum : uint32_t { ST_TAPE_TIMEOUT = 1u, ST_TAPE_CORRUPT = 2u };

#ifndef __CUDACC_RTC__
// Kernel kinds the launch log attributes device time to.
// (the primary level's march / AO / shadow passes apart from the reflection levels').
enum KernelKind : uint32_t {
    KK_MARCH = 0, KK_AO, KK_SHADOW, KK_SHADE, KK_RESOLVE, KK_POST, KK_AOV, KK_GI, KK_OTHER,
    KK_MARCH_REFL, KK_AO_REFL, KK_SHADOW_REFL, KK_COUNT
};

// Counts launches and, when a recorder is attached, brackets each with CUDA events.
struct LaunchLog {
    uint32_t launches = 0;
    void* recorder = nullptr;  // opaque (the context's profiler)
    void (*begin)(void* recorder, uint32_t kind, cudaStream_t s) = nullptr;
    void (*end)(void* recorder, uint32_t kind, cudaStream_t s) = nullptr;
};

// Launch-log bracket of one pass: counts its `n` launches and brackets it for the recorder.
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

// Kernels of a scene-specialised program (NVRTC, see spec.h): the march / shadow / AO passes
// with the scene's field compiled in; same parameters as the library's kernels.
struct SpecKernels {
    const void* march = nullptr;
    const void* shadow = nullptr;
    const void* ao = nullptr;
    uint32_t block = 128;   // threads per CTA they were compiled for
    bool smem_tape = true;  // they stage the tape in shared memory
};

// With `spec`, the pass runs the specialised kernel instead of the interpreter.
cudaError_t launch_march(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log,
                         const SpecKernels* spec = nullptr);
cudaError_t launch_ao(const WaveArgs& a, cudaStream_t s, LaunchLog* log, const SpecKernels* spec = nullptr);
cudaError_t launch_shadow(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log,
                          const SpecKernels* spec = nullptr);
cudaError_t launch_shade(const WaveArgs& a, cudaStream_t s, LaunchLog* log);
// Reflection rays of the level's hits (the rays shade would append), into the next queue.
cudaError_t launch_reflect(const WaveArgs& a, cudaStream_t s, LaunchLog* log);
// Pixel slots of the jobs (n_slots when known on the host, else capacity + a.totals).
cudaError_t launch_resolve(const WaveArgs& a, uint32_t n_slots, cudaStream_t s, LaunchLog* log);
// AOV modes: display value per pixel-centre hit of job 0 (lib.rs:1185-1217), written as RGBA f32.
cudaError_t launch_aov(const WaveArgs& a, float4* out, cudaStream_t s, LaunchLog* log);
// GI gather shading: emissive + unshadowed direct light at each gather hit (lib.rs:686-711).
cudaError_t launch_gather_shade(const WaveArgs& a, float4* radiance, cudaStream_t s, LaunchLog* log);

// Post stack (post.rs:36-115) over the output pixels of the jobs: bright-pass, separable
// Gaussian (per-job weights), add, exposure, ACES, gamma, clamp; RGBA f32 or RGBA8 into
// each job's `out`. With bloom it is two launches: bright-pass + horizontal blur into
// `blur_h`, then vertical blur + resolve.
struct PostArgs {
    FrameJob job0;
    const FrameJob* jobs;
    const JobTotals* totals;
    uint32_t n_jobs;
    uint32_t n_pixels;  // output pixels when known on the host, else capacity
    int any_bloom;      // some job blooms
    uint32_t grid_cap;  // block limit of the grid-stride kernels (0: one thread per pixel)
    const float4* hdr;
    float4* blur_h;  // horizontal blur of the bright-pass (one float4 per output pixel)
};
cudaError_t launch_post(const PostArgs& p, cudaStream_t s, LaunchLog* log);
cudaError_t launch_pack_rgba8(const float4* src, uchar4* dst, size_t n, cudaStream_t s, LaunchLog* log);
cudaError_t launch_field(const unsigned char* tape, const float* pts, uint32_t n, float* dist, uint32_t* mat,
                         cudaStream_t s, LaunchLog* log);
cudaError_t launch_gi_reduce(const float4* radiance, const float4* dirs, uint32_t dirs_per_face, uint32_t probes,
                             float4* cubes, cudaStream_t s, LaunchLog* log);

// G-buffer and reprojection passes (reproject.cu).
// G-buffer pixels of an aa-1 frame from its primary-level records and resolved HDR.
cudaError_t launch_gbuffer_pack(const WaveArgs& a, uint32_t n_slots, const float4* movers, uint32_t n_movers,
                                uchar4* color, float* depth, int32_t* obj, cudaStream_t s, LaunchLog* log);
// Forward warp: per target pixel the nearest source (keys: scratch of w*h 64-bit words).
cudaError_t launch_warp(const CameraArgs& prev, const CameraArgs& next, uint32_t w, uint32_t h, const float* depth,
                        const int32_t* obj, const float* deltas3, uint32_t n_deltas, unsigned long long* keys,
                        const uchar4* src, uchar4* out, unsigned char* filled, cudaStream_t s, LaunchLog* log);
cudaError_t launch_row_fill(uint32_t w, uint32_t h, uchar4* out, unsigned char* filled, cudaStream_t s,
                            LaunchLog* log);
// Holes of `filled` as a primary ray queue (q_o / q_d, *count, hole_pix); *count must start at 0.
cudaError_t launch_hole_rays(const CameraArgs& cam, uint32_t w, uint32_t h, const unsigned char* filled, float4* q_o,
                             float4* q_d, uint32_t* hole_pix, uint32_t* count, uint32_t grid_cap, cudaStream_t s,
                             LaunchLog* log);
// Display pixel of every shaded hole (its levels folded), written at hole_pix.
cudaError_t launch_hole_resolve(const WaveArgs& a, const uint32_t* count, const uint32_t* hole_pix, uchar4* out,
                                cudaStream_t s, LaunchLog* log);

#endif  // __CUDACC_RTC__

}  // namespace mm3e
