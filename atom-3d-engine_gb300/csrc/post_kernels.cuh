// post_kernels.cuh — the post kernels of the render path (post.rs:36-115: bright-pass, separable
// Gaussian bloom, exposure, ACES, gamma and the framebuffer write) over the output pixels of
// every job of a pass sequence. Their launcher is launch_post in wavefront.cu.
#pragma once
#include "../../include/mm3e_cuda.h"
#include "kernels.h"
#include "march_kernels.cuh"

namespace mm3e {
namespace wave {

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

}  // namespace wave
}  // namespace mm3e
