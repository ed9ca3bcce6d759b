// wavefront.cu — sm_103a wavefront kernels of the MM3E per-pixel SDF render path.
//
// A frame is a short sequence of small kernels over ray queues. Keeping each kernel's code
// footprint small matters more here than anything else: a single kernel holding the march,
// the shadow march, AO and all of the shading stalls on instruction fetch. The march,
// shadow and AO bodies live in march_kernels.cuh (shared with the scene-specialised NVRTC
// program), and the per-slot shading, reflection-emit and resolve bodies in shade_kernels.cuh.
// This file instantiates them as kernels (the field passes with the tape interpreter) and holds
// the AOV, GI and post kernels.
#include <cuda_runtime.h>

#include "../../include/mm3e_cuda.h"
#include "kernels.h"
#include "march_kernels.cuh"
#include "shade_kernels.cuh"

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

// ---------------------------------------------------------------------------------------
// Post (post.rs:36-115), over the output pixels of every job of the pass sequence
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t post_pixels(const PostArgs& p) { return p.jobs ? p.totals->n_pixels : p.n_pixels; }
__device__ __forceinline__ const FrameJob* post_job(const PostArgs& p, uint32_t i) {
    return p.jobs ? &p.jobs[find_job<2>(p.jobs, p.totals->n_jobs, i)] : &p.job0;
}
#define MM3E_POST_LOOP(i, p)                                              \
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, n_ = post_pixels(p); i < n_; \
         i += gridDim.x * blockDim.x)

// Bright-pass of one pixel (post.rs:64-69).
__device__ __forceinline__ V bright_of(const PostArgs& p, const FrameJob* J, uint32_t i) {
    float4 c = p.hdr[i];
    V v{c.x, c.y, c.z};
    float l = luminance(v);
    float thr = J->threshold;
    V b{0.f, 0.f, 0.f};
    if (l > thr) b = scale(v, (l - thr) / fmaxf(l, 1e-4f));
    return b;
}

// Four outputs of one separable Gaussian pass (post.rs:348-368) that lie next to each other
// along the blur axis. Their taps overlap, so each source pixel is read once for all four:
// tap(j), j = 0 .. 2r+3, is the clamped source pixel at offset j - r from output 0, and output o
// takes it with weight kw[j - o]. Every output sums its 2r+1 taps in kernel order from zero, as
// the one-output loop does, so the sums are the same floats. Needs r >= 1 (the reference blurs
// with at least radius 1).
template <class TAP>
__device__ __forceinline__ void blur4(const float* __restrict__ kw, int r, TAP tap, V& a0, V& a1, V& a2, V& a3) {
    a0 = a1 = a2 = a3 = V{0.f, 0.f, 0.f};
    const float k0 = __ldg(kw), k1 = __ldg(kw + 1), k2 = __ldg(kw + 2);
    V v = tap(0);
    a0 = a0 + scale(v, k0);
    v = tap(1);
    a0 = a0 + scale(v, k1);
    a1 = a1 + scale(v, k0);
    v = tap(2);
    a0 = a0 + scale(v, k2);
    a1 = a1 + scale(v, k1);
    a2 = a2 + scale(v, k0);
    float c1 = k2, c2 = k1, c3 = k0;  // kw[j-1], kw[j-2], kw[j-3] at the top of step j
#pragma unroll 4
    for (int j = 3; j <= 2 * r; ++j) {
        const float c0 = __ldg(kw + j);
        v = tap(j);
        a0 = a0 + scale(v, c0);
        a1 = a1 + scale(v, c1);
        a2 = a2 + scale(v, c2);
        a3 = a3 + scale(v, c3);
        c3 = c2;
        c2 = c1;
        c1 = c0;
    }
    v = tap(2 * r + 1);
    a1 = a1 + scale(v, c1);
    a2 = a2 + scale(v, c2);
    a3 = a3 + scale(v, c3);
    v = tap(2 * r + 2);
    a2 = a2 + scale(v, c1);
    a3 = a3 + scale(v, c2);
    v = tap(2 * r + 3);
    a3 = a3 + scale(v, c1);
}

// Bright-pass fused with the horizontal blur. A block takes BLOOM_SEG consecutive output pixels
// at a time (four per thread), with their bright-pass values and a halo of BLOOM_HALO pixels
// on either side computed once into shared memory. A thread whose four pixels share one row of
// a blooming job and whose radius fits the halo blurs them together (blur4); any other pixel
// sums its own taps, computing the bright-pass of a tap outside the window on the spot.
// Window element e sits at slot e ^ ((e / 8) % 4): the eight threads of a quarter warp read
// elements four apart, which this swizzle (a permutation within each run of eight 16-byte
// slots) spreads over all 32 banks, so a warp's read takes the minimum four wavefronts.
constexpr int BLOOM_SEG = POST_THREADS * 4;
constexpr int BLOOM_HALO = 32;
constexpr int BLOOM_WIN = BLOOM_SEG + 2 * BLOOM_HALO;
static_assert(BLOOM_WIN % 8 == 0, "the window swizzle permutes runs of eight slots");
__device__ __forceinline__ int win_slot(int e) { return e ^ ((e >> 3) & 3); }

__global__ void __launch_bounds__(POST_THREADS) k_bloom_h(const __grid_constant__ PostArgs p) {
    __shared__ float4 win[BLOOM_WIN];  // BLOOM_WIN is a multiple of 8
    const uint32_t n = post_pixels(p);
    for (uint32_t seg = blockIdx.x * (uint32_t)BLOOM_SEG; seg < n; seg += gridDim.x * (uint32_t)BLOOM_SEG) {
        const long long lo = (long long)seg - BLOOM_HALO;
        for (int e = threadIdx.x; e < BLOOM_WIN; e += POST_THREADS) {
            const long long g = lo + e;
            V b{0.f, 0.f, 0.f};
            if (g >= 0 && g < (long long)n) {
                const FrameJob* J = post_job(p, (uint32_t)g);
                if (J->flags & JF_BLOOM) b = bright_of(p, J, (uint32_t)g);
            }
            win[win_slot(e)] = make_float4(b.x, b.y, b.z, 0.0f);
        }
        __syncthreads();
        const uint32_t i0 = seg + 4u * threadIdx.x;
        if (i0 < n) {
            const FrameJob* J = post_job(p, i0);
            const uint32_t w = J->width, local = i0 - J->pixel_base;
            const uint32_t x0 = local % w, y = local / w;
            const int r = (int)J->bloom_radius;
            const long long row_e = (long long)J->pixel_base + (long long)y * w - lo;  // window index of the row's x = 0
            if ((J->flags & JF_BLOOM) && x0 + 3u < w && r >= 1 && r <= BLOOM_HALO) {
                const int xl = (int)x0 - r, xmax = (int)w - 1;
                auto tap = [&](int j) {
                    const float4 s = win[win_slot((int)(row_e + min(max(xl + j, 0), xmax)))];
                    return V{s.x, s.y, s.z};
                };
                V a0, a1, a2, a3;
                blur4(J->bloom_w, r, tap, a0, a1, a2, a3);
                p.blur_h[i0] = make_float4(a0.x, a0.y, a0.z, 0.0f);
                p.blur_h[i0 + 1] = make_float4(a1.x, a1.y, a1.z, 0.0f);
                p.blur_h[i0 + 2] = make_float4(a2.x, a2.y, a2.z, 0.0f);
                p.blur_h[i0 + 3] = make_float4(a3.x, a3.y, a3.z, 0.0f);
            } else {
                for (uint32_t i = i0; i < i0 + 4u && i < n; ++i) {
                    const FrameJob* Ji = post_job(p, i);
                    if (!(Ji->flags & JF_BLOOM)) continue;
                    const uint32_t wi = Ji->width, li = i - Ji->pixel_base;
                    const int x = (int)(li % wi), ri = (int)Ji->bloom_radius;
                    const uint32_t row = Ji->pixel_base + (li / wi) * wi;
                    V acc{0.f, 0.f, 0.f};
                    for (int ki = 0; ki <= 2 * ri; ++ki) {
                        const uint32_t g = row + (uint32_t)min(max(x + ki - ri, 0), (int)wi - 1);
                        const long long e = (long long)g - lo;
                        V v;
                        if (e >= 0 && e < BLOOM_WIN) {
                            const float4 s = win[win_slot((int)e)];
                            v = V{s.x, s.y, s.z};
                        } else {
                            v = bright_of(p, Ji, g);
                        }
                        acc = acc + scale(v, __ldg(Ji->bloom_w + ki));
                    }
                    p.blur_h[i] = make_float4(acc.x, acc.y, acc.z, 0.0f);
                }
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ unsigned char to_u8(float c) {
    return (unsigned char)__float2uint_rz(clampf(c, 0.0f, 1.0f) * 255.0f + 0.5f);
}

// Bloom add, exposure, ACES, gamma and the framebuffer write of one pixel (post.rs:40-55).
__device__ __forceinline__ void resolve_pixel(const PostArgs& p, const FrameJob* J, uint32_t i, bool bloom, V blurred) {
    float4 c = p.hdr[i];
    V col{c.x, c.y, c.z};
    if (bloom) col = col + scale(blurred, J->intensity);
    V d = display(col, J->exposure);
    uint32_t local = i - J->pixel_base;
    if (J->format == MM3E_FB_RGBA8)
        reinterpret_cast<uchar4*>(J->out)[local] = make_uchar4(to_u8(d.x), to_u8(d.y), to_u8(d.z), 255);
    else reinterpret_cast<float4*>(J->out)[local] = make_float4(d.x, d.y, d.z, 1.0f);
}

// Post without bloom: resolve only.
__global__ void __launch_bounds__(POST_THREADS) k_resolve_post(const __grid_constant__ PostArgs p) {
    MM3E_POST_LOOP(i, p) {
        const FrameJob* J = post_job(p, i);
        if (J->out) resolve_pixel(p, J, i, false, V{0.f, 0.f, 0.f});
    }
}

// Vertical blur of the horizontal pass fused with the resolve. One frame: a thread takes four
// rows of one column (blur4 over the column's taps, read through L1). Several jobs: one pixel
// per thread, its own taps.
template <bool ONE_JOB>
__global__ void __launch_bounds__(POST_THREADS) k_bloom_v(const __grid_constant__ PostArgs p) {
    if constexpr (ONE_JOB) {
        const FrameJob* J = &p.job0;
        if (!J->out) return;
        const uint32_t w = J->width, h = J->height, groups = w * ((h + 3u) / 4u);
        const bool bloom = (J->flags & JF_BLOOM) != 0;
        const int r = (int)J->bloom_radius, ymax = (int)h - 1;
        const float4* img = p.blur_h + J->pixel_base;
        for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += gridDim.x * blockDim.x) {
            const uint32_t x = g % w, y0 = (g / w) * 4u;
            V a0{0.f, 0.f, 0.f}, a1 = a0, a2 = a0, a3 = a0;
            if (bloom) {
                const int yl = (int)y0 - r;
                auto tap = [&](int j) {
                    const float4 s = __ldg(img + (size_t)min(max(yl + j, 0), ymax) * w + x);
                    return V{s.x, s.y, s.z};
                };
                blur4(J->bloom_w, r, tap, a0, a1, a2, a3);
            }
            const uint32_t i = J->pixel_base + y0 * w + x;
            resolve_pixel(p, J, i, bloom, a0);
            if (y0 + 1u < h) resolve_pixel(p, J, i + w, bloom, a1);
            if (y0 + 2u < h) resolve_pixel(p, J, i + 2u * w, bloom, a2);
            if (y0 + 3u < h) resolve_pixel(p, J, i + 3u * w, bloom, a3);
        }
    } else {
        MM3E_POST_LOOP(i, p) {
            const FrameJob* J = post_job(p, i);
            if (!J->out) continue;
            if (!(J->flags & JF_BLOOM)) {
                resolve_pixel(p, J, i, false, V{0.f, 0.f, 0.f});
                continue;
            }
            const uint32_t w = J->width, h = J->height, local = i - J->pixel_base;
            const int x = (int)(local % w), y = (int)(local / w), r = (int)J->bloom_radius;
            const float4* img = p.blur_h + J->pixel_base;
            V acc{0.f, 0.f, 0.f};
            for (int ki = 0; ki <= 2 * r; ++ki) {
                const float4 s = __ldg(img + (size_t)min(max(y + ki - r, 0), (int)h - 1) * w + x);
                acc = acc + scale(V{s.x, s.y, s.z}, __ldg(J->bloom_w + ki));
            }
            resolve_pixel(p, J, i, true, acc);
        }
    }
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
