// wavefront.cu — sm_103a wavefront kernels of the MM3E per-pixel SDF render path.
//
// A frame is a short sequence of small kernels over ray queues. Keeping each kernel's code
// footprint small matters more here than anything else: a single kernel holding the march,
// the shadow march, AO and all of the shading stalls on instruction fetch. The march,
// shadow and AO bodies live in march_kernels.cuh (shared with the scene-specialised NVRTC
// program), the per-slot shading, reflection-emit, resolve, AOV and GI bodies in
// shade_kernels.cuh, and the post kernels in post_kernels.cuh. This file instantiates the passes
// as kernels (the field passes with the tape interpreter) and launches them.
#include <cuda_runtime.h>

#include "../../include/mm3e_cuda.h"
#include "kernels.h"
#include "march_kernels.cuh"
#include "shade_kernels.cuh"
#include "post_kernels.cuh"

namespace mm3e {
namespace {

using namespace wave;

template <int TM, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) k_march(const __grid_constant__ WaveArgs a) {
    march_body<TM, UNROLL, InterpField>(a);
}

template <int TM, int BLOCK, int UNROLL>
__global__ void __launch_bounds__(BLOCK) k_shadow(const __grid_constant__ WaveArgs a) {
    shadow_body<TM, UNROLL, InterpField>(a);
}

__global__ void __launch_bounds__(SHADE_THREADS) k_ao(const __grid_constant__ WaveArgs a) { ao_body<InterpField>(a); }

__global__ void __launch_bounds__(SHADE_THREADS) k_shade(const __grid_constant__ WaveArgs a) {
    if (pass_failed(a)) return;
    const uint32_t n = item_count(a);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
        shade_slots(a, base + threadIdx.x, base + threadIdx.x < n);  // block-uniform trip count
}

__global__ void __launch_bounds__(SHADE_THREADS) k_reflect(const __grid_constant__ WaveArgs a) {
    if (pass_failed(a)) return;
    const uint32_t n = item_count(a);
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
        reflect_slots(a, base + threadIdx.x, base + threadIdx.x < n);
}

__global__ void __launch_bounds__(SHADE_THREADS) k_resolve(const __grid_constant__ WaveArgs a, uint32_t n_slots) {
    if (pass_failed(a)) return;
    uint32_t nj = 1;
    if (a.jobs) {
        n_slots = a.totals->n_slots;
        nj = a.totals->n_jobs;
    }
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n_slots; slot += gridDim.x * blockDim.x)
        resolve_slot(a, slot, nj);
}

// AOV display values (lib.rs:1185-1217) for pixel-centre hits of job 0 (row-major slots).
__global__ void __launch_bounds__(SHADE_THREADS) k_aov(const __grid_constant__ WaveArgs a, float4* out) {
    if (pass_failed(a)) return;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot < a.job0.width * a.job0.height) aov_slot(a, slot, out);
}

// Scene::gather (lib.rs:686-711) at every gather ray's hit.
__global__ void __launch_bounds__(SHADE_THREADS) k_gather_shade(const __grid_constant__ WaveArgs a, float4* radiance) {
    if (pass_failed(a)) return;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot < a.n_items) gather_slot(a, slot, radiance);
}

__global__ void k_pack8(const float4* __restrict__ src, uchar4* __restrict__ dst, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 c = src[i];
    dst[i] = make_uchar4(to_u8(c.x), to_u8(c.y), to_u8(c.z), 255);
}

__global__ void k_field(const unsigned char* __restrict__ tape, const float* __restrict__ pts, uint32_t n,
                        float* __restrict__ dist, uint32_t* __restrict__ mat) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Tape T = tape_view(tape);
    Field f = world_eval(T, V{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    dist[i] = f.d;
    mat[i] = f.m;
}

// GiVolume::bake per-face average (gi.rs:78-86), one thread per probe face.
__global__ void k_gi_reduce(const float4* __restrict__ rad, const float4* __restrict__ dirs, uint32_t dpf,
                            uint32_t probes, float4* __restrict__ cubes) {
    uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;  // probe*6 + face
    if (idx < probes * 6u) gi_reduce_slot(rad, dirs, dpf, idx, cubes);
}

typedef void (*WaveKernel)(const WaveArgs);

// Instantiations of a persistent kernel over (tape mode, block, unroll).
// Samples a lane steps between refills: the tuning's unroll rounded down to 1, 16 or 64. Long
// runs keep the warp in the step loop, whose field code then stays in the instruction cache
// (measured: 32 to 64 samples per refill cut the specialised frame times by 30-45%).
constexpr int unroll_index(uint32_t u) { return u >= 64 ? 2 : (u >= 16 ? 1 : 0); }

struct PersistentSet {
    WaveKernel k[2][2][3];  // [tape mode][block 128 / 256][unroll 1 / 16 / 64]
};

#define MM3E_PERSISTENT_SET(K)                                                                             \
    PersistentSet {                                                                                        \
        {{{K<TM_SMEM, 128, 1>, K<TM_SMEM, 128, 16>, K<TM_SMEM, 128, 64>},                                  \
          {K<TM_SMEM, 256, 1>, K<TM_SMEM, 256, 16>, K<TM_SMEM, 256, 64>}},                                 \
         {{K<TM_MULTI, 128, 1>, K<TM_MULTI, 128, 16>, K<TM_MULTI, 128, 64>},                               \
          {K<TM_MULTI, 256, 1>, K<TM_MULTI, 256, 16>, K<TM_MULTI, 256, 64>}}}                              \
    }

// Grid of a persistent launch: every CTA the SMs hold at once, fewer when the host knows
// that fewer items exist.
cudaError_t persistent_grid(const void* k, int block, size_t smem, const WaveArgs& a, int sm_count,
                            uint32_t items_per_item, uint32_t* blocks_out) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint32_t blocks = (uint32_t)(per_sm * sm_count);
    if (!a.n_items_dev) {
        uint64_t items = (uint64_t)a.n_items * items_per_item;
        uint64_t needed = (items + block - 1) / block;
        if (needed < blocks) blocks = needed > 0 ? (uint32_t)needed : 1u;
    }
    *blocks_out = blocks;
    return cudaSuccess;
}

cudaError_t launch_persistent(const PersistentSet& set, const WaveArgs& a, const TuneParams& t, cudaStream_t s,
                              int sm_count, uint32_t items_per_item) {
    bool use_smem = !a.jobs && a.tape_bytes <= SMEM_TAPE_MAX;
    int bi = t.block >= 256 ? 1 : 0;
    int ui = unroll_index(t.unroll);
    int block = bi ? 256 : 128;
    WaveKernel k = set.k[use_smem ? 0 : 1][bi][ui];
    size_t smem = use_smem ? a.tape_bytes : 0;
    if (use_smem && smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TAPE_MAX);
        if (e != cudaSuccess) return e;
    }
    uint32_t blocks = 0;
    cudaError_t e = persistent_grid(reinterpret_cast<const void*>(k), block, smem, a, sm_count, items_per_item, &blocks);
    if (e != cudaSuccess) return e;
    k<<<blocks, block, smem, s>>>(a);
    return cudaGetLastError();
}

// A specialised (run-time compiled) persistent kernel.
cudaError_t launch_persistent_spec(const void* k, const SpecKernels& sp, const WaveArgs& a, cudaStream_t s,
                                   int sm_count, uint32_t items_per_item) {
    size_t smem = sp.smem_tape ? a.tape_bytes : 0;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TAPE_MAX);
        if (e != cudaSuccess) return e;
    }
    uint32_t blocks = 0;
    cudaError_t e = persistent_grid(k, (int)sp.block, smem, a, sm_count, items_per_item, &blocks);
    if (e != cudaSuccess) return e;
    WaveArgs arg = a;
    void* args[] = {&arg};
    return cudaLaunchKernel(k, dim3(blocks), dim3(sp.block), args, smem, s);
}

unsigned grid_for(uint64_t n, int threads, uint32_t cap = 0) {
    uint64_t g = (n + threads - 1) / threads;
    if (cap && g > cap) g = cap;
    return g > 0 ? (unsigned)g : 1u;
}

}  // namespace

cudaError_t launch_march(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log,
                         const SpecKernels* spec) {
    static const PersistentSet set = MM3E_PERSISTENT_SET(k_march);
    LogScope sc(log, a.level == 0 ? KK_MARCH : KK_MARCH_REFL, s, 1);
    if (spec && spec->march && !a.jobs) return launch_persistent_spec(spec->march, *spec, a, s, sm_count, 1);
    return launch_persistent(set, a, t, s, sm_count, 1);
}

cudaError_t launch_shadow(const WaveArgs& a, const TuneParams& t, cudaStream_t s, int sm_count, LaunchLog* log,
                          const SpecKernels* spec) {
    static const PersistentSet set = MM3E_PERSISTENT_SET(k_shadow);
    LogScope sc(log, a.level == 0 ? KK_SHADOW : KK_SHADOW_REFL, s, 1);
    uint32_t per = a.lights_max ? a.lights_max : 1;
    if (spec && spec->shadow && !a.jobs) return launch_persistent_spec(spec->shadow, *spec, a, s, sm_count, per);
    return launch_persistent(set, a, t, s, sm_count, per);
}

// Non-persistent kernels are sized for the largest queue (a.n_items) and read the live count
// from n_items_dev when set.
cudaError_t launch_ao(const WaveArgs& a, cudaStream_t s, LaunchLog* log, const SpecKernels* spec) {
    LogScope sc(log, a.level == 0 ? KK_AO : KK_AO_REFL, s, 1);
    unsigned grid = grid_for(a.n_items, SHADE_THREADS, a.grid_cap);
    if (spec && spec->ao && !a.jobs) {
        WaveArgs arg = a;
        void* args[] = {&arg};
        return cudaLaunchKernel(spec->ao, dim3(grid), dim3(SHADE_THREADS), args, 0, s);
    }
    k_ao<<<grid, SHADE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_shade(const WaveArgs& a, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_SHADE, s, 1);
    k_shade<<<grid_for(a.n_items, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_reflect(const WaveArgs& a, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_SHADE, s, 1);
    k_reflect<<<grid_for(a.n_items, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const WaveArgs& a, uint32_t n_slots, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_RESOLVE, s, 1);
    k_resolve<<<grid_for(n_slots, SHADE_THREADS, a.grid_cap), SHADE_THREADS, 0, s>>>(a, n_slots);
    return cudaGetLastError();
}

cudaError_t launch_aov(const WaveArgs& a, float4* out, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_AOV, s, 1);
    k_aov<<<grid_for((uint64_t)a.job0.width * a.job0.height, SHADE_THREADS), SHADE_THREADS, 0, s>>>(a, out);
    return cudaGetLastError();
}

cudaError_t launch_gather_shade(const WaveArgs& a, float4* radiance, cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_GI, s, 1);
    k_gather_shade<<<grid_for(a.n_items, SHADE_THREADS), SHADE_THREADS, 0, s>>>(a, radiance);
    return cudaGetLastError();
}

cudaError_t launch_post(const PostArgs& p, cudaStream_t s, LaunchLog* log) {
    if (p.n_pixels == 0) return cudaSuccess;
    LogScope sc(log, KK_POST, s, p.any_bloom ? 2u : 1u);
    if (!p.any_bloom) {
        k_resolve_post<<<grid_for(p.n_pixels, POST_THREADS, p.grid_cap), POST_THREADS, 0, s>>>(p);
        return cudaGetLastError();
    }
    k_bloom_h<<<grid_for(((uint64_t)p.n_pixels + BLOOM_SEG - 1) / BLOOM_SEG, 1, p.grid_cap), POST_THREADS, 0, s>>>(p);
    if (p.jobs) {
        k_bloom_v<false><<<grid_for(p.n_pixels, POST_THREADS, p.grid_cap), POST_THREADS, 0, s>>>(p);
    } else {
        const uint64_t groups = (uint64_t)p.job0.width * ((p.job0.height + 3u) / 4u);
        k_bloom_v<true><<<grid_for(groups, POST_THREADS, p.grid_cap), POST_THREADS, 0, s>>>(p);
    }
    return cudaGetLastError();
}

cudaError_t launch_pack_rgba8(const float4* src, uchar4* dst, size_t n, cudaStream_t s, LaunchLog* log) {
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 1);
    k_pack8<<<grid_for(n, POST_THREADS), POST_THREADS, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_field(const unsigned char* tape, const float* pts, uint32_t n, float* dist, uint32_t* mat,
                         cudaStream_t s, LaunchLog* log) {
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 1);
    k_field<<<grid_for(n, 128), 128, 0, s>>>(tape, pts, n, dist, mat);
    return cudaGetLastError();
}

cudaError_t launch_gi_reduce(const float4* radiance, const float4* dirs, uint32_t dirs_per_face, uint32_t probes,
                             float4* cubes, cudaStream_t s, LaunchLog* log) {
    uint32_t n = probes * 6u;
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_GI, s, 1);
    k_gi_reduce<<<grid_for(n, 128), 128, 0, s>>>(radiance, dirs, dirs_per_face, probes, cubes);
    return cudaGetLastError();
}

}  // namespace mm3e
