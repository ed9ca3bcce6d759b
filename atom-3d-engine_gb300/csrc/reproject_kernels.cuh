// reproject_kernels.cuh — kernels of the preview path: G-buffer packing and camera
// reprojection (mm3e-orchestrator/src/lib.rs:951-1080, reproject.rs:55-146). Their launchers are
// in reproject.cu. Every kernel is a grid-stride loop over its items, so a single thread runs all
// of them in scan order as well.
//
// The forward warp keeps, per target pixel, the nearest source point as the reference's
// sequential z-buffer does: one 64-bit atomicMin per source pixel on (forward depth bits,
// source index), so equal depths resolve to the earliest source in scan order, exactly as
// the reference's strict `fz < zbuf` test in row-major order.
#pragma once
#include "kernels.h"
#include "march_kernels.cuh"

namespace mm3e {
namespace preview {

using namespace wave;

constexpr int RP_THREADS = 256;

__device__ __forceinline__ unsigned char u8_of(float c) {  // (c * 255 + 0.5) as u8 after clamp01
    return (unsigned char)__float2uint_rz(c * 255.0f + 0.5f);
}

// render_gbuffer's pixel (lib.rs:988-1018) from the primary level's records of an aa-1 frame.
__global__ void __launch_bounds__(RP_THREADS)
    k_gbuffer_pack(const __grid_constant__ WaveArgs a, uint32_t n_slots, const float4* __restrict__ movers,
                   uint32_t n_movers, uchar4* __restrict__ color, float* __restrict__ depth, int32_t* __restrict__ obj) {
    const FrameJob& J = a.job0;
    const TapeHeader* h = reinterpret_cast<const TapeHeader*>(J.tape);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_slots; p += gridDim.x * blockDim.x) {
        uint32_t x, y;
        if (!tiled_pixel(p, J, a.tile_wlog, x, y)) continue;
        size_t i = (size_t)y * J.width + x;
        float4 c = a.b.hdr[i];
        V d = display(V{c.x, c.y, c.z}, h->exposure);
        color[i] = make_uchar4(u8_of(d.x), u8_of(d.y), u8_of(d.z), 255);
        uint2 hm = a.b.h_m[p];
        if (hm.x == NIL) {
            depth[i] = __int_as_float(0x7f800000);
            obj[i] = -1;
            continue;
        }
        float4 hn4 = a.b.h_n[p], o4 = a.b.q_o[p], d4 = a.b.q_d[p];
        V pos = V{o4.x, o4.y, o4.z} + scale(V{d4.x, d4.y, d4.z}, hn4.w);
        int32_t o = -1;
        for (uint32_t k = 0; k < n_movers; ++k) {
            float4 m = movers[k];
            if (length(pos - V{m.x, m.y, m.z}) <= m.w + 0.05f) {
                o = (int32_t)k;
                break;
            }
        }
        depth[i] = hn4.w;
        obj[i] = o;
    }
}

// reproject.rs:55-70
__device__ __forceinline__ bool project(const CameraArgs& c, V world, uint32_t w, uint32_t h, float& sx, float& sy,
                                        float& fz) {
    V v = world - ld3(c.eye);
    fz = dot(v, ld3(c.fwd));
    if (fz <= 1e-4f) return false;
    float aspect = (float)w / (float)h;
    float ndc_x = dot(v, ld3(c.right)) / fz;
    float ndc_y = dot(v, ld3(c.up)) / fz;
    sx = (ndc_x / (aspect * c.fov_scale) + 1.0f) * 0.5f * (float)w;
    sy = (1.0f - ndc_y / c.fov_scale) * 0.5f * (float)h;
    return true;
}

// reproject.rs:77-113, first half: the nearest source of every target pixel.
__global__ void __launch_bounds__(RP_THREADS)
    k_warp_keys(CameraArgs prev, CameraArgs next, uint32_t w, uint32_t h, const float* __restrict__ depth,
                const int32_t* __restrict__ obj, const float* __restrict__ deltas3, uint32_t n_deltas,
                unsigned long long* __restrict__ keys) {
    size_t n = (size_t)w * h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)(i % w), y = (uint32_t)(i / w);
        V dir = camera_dir(prev, (float)x + 0.5f, (float)y + 0.5f, w, h);
        float d = isfinite(depth[i]) ? depth[i] : 1.0e6f;
        V world = ld3(prev.eye) + scale(dir, d);
        int32_t oi = obj[i];
        if (oi >= 0 && (uint32_t)oi < n_deltas)
            world = world + V{deltas3[3 * oi], deltas3[3 * oi + 1], deltas3[3 * oi + 2]};
        float sx, sy, fz;
        // a NaN or infinite depth never beats the z-buffer's initial +inf in the sequential test
        if (!project(next, world, w, h, sx, sy, fz) || !(fz < __int_as_float(0x7f800000))) continue;
        int32_t nx = (int32_t)floorf(sx), ny = (int32_t)floorf(sy);
        if (nx < 0 || ny < 0 || (uint32_t)nx >= w || (uint32_t)ny >= h) continue;
        unsigned long long key = ((unsigned long long)__float_as_uint(fz) << 32) | (unsigned long long)i;
        atomicMin(&keys[(size_t)ny * w + nx], key);
    }
}

__global__ void __launch_bounds__(RP_THREADS)
    k_warp_apply(uint32_t n, const unsigned long long* __restrict__ keys, const uchar4* __restrict__ src,
                 uchar4* __restrict__ out, unsigned char* __restrict__ filled) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        unsigned long long k = keys[j];
        bool f = k != ~0ull;
        out[j] = f ? src[(uint32_t)(k & 0xFFFFFFFFull)] : make_uchar4(0, 0, 0, 0);
        filled[j] = f ? 1 : 0;
    }
}

// reproject.rs:118-146: each unfilled pixel takes the last filled pixel on its row, then the
// row's leading edge takes the first; one thread per row.
__global__ void k_row_fill(uint32_t w, uint32_t h, uchar4* __restrict__ out, unsigned char* __restrict__ filled) {
    uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= h) return;
    uchar4* row = out + (size_t)y * w;
    unsigned char* fr = filled + (size_t)y * w;
    bool have = false;
    uchar4 last = make_uchar4(0, 0, 0, 0);
    for (uint32_t x = 0; x < w; ++x) {
        if (fr[x]) {
            last = row[x];
            have = true;
        } else if (have) {
            row[x] = last;
            fr[x] = 1;
        }
    }
    have = false;
    for (uint32_t x = w; x-- > 0;) {
        if (fr[x]) {
            last = row[x];
            have = true;
        } else if (have) {
            row[x] = last;
        }
    }
}

// reproject_hybrid (lib.rs:1050-1078): the new camera's ray of every hole, queued for the
// primary level (sample k of the queue is hole k; hole_pix[k] is its pixel).
__global__ void __launch_bounds__(RP_THREADS)
    k_hole_rays(CameraArgs cam, uint32_t w, uint32_t h, const unsigned char* __restrict__ filled, float4* __restrict__ q_o,
                float4* __restrict__ q_d, uint32_t* __restrict__ hole_pix, uint32_t* __restrict__ count) {
    const uint32_t n = w * h;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        uint32_t j = base + threadIdx.x;
        bool hole = j < n && !filled[j];
        const uint32_t lane = threadIdx.x & 31u;
        unsigned mask = __ballot_sync(0xFFFFFFFFu, hole);
        if (!mask) continue;
        uint32_t b = 0;
        int leader = __ffs(mask) - 1;
        if ((int)lane == leader) b = atomicAdd(count, (uint32_t)__popc(mask));
        b = __shfl_sync(0xFFFFFFFFu, b, leader);
        if (hole) {
            uint32_t k = b + (uint32_t)__popc(mask & ((1u << lane) - 1u));
            uint32_t x = j % w, y = j / w;
            V d = camera_dir(cam, (float)x + 0.5f, (float)y + 0.5f, w, h);
            q_o[k] = make_float4(cam.eye[0], cam.eye[1], cam.eye[2], __uint_as_float(k));
            q_d[k] = make_float4(d.x, d.y, d.z, 0.0f);
            hole_pix[k] = j;
        }
    }
}

// Each hole's radiance (its levels folded as k_resolve does for one sample) as a display pixel.
__global__ void __launch_bounds__(RP_THREADS)
    k_hole_resolve(const __grid_constant__ WaveArgs a, const uint32_t* __restrict__ count,
                   const uint32_t* __restrict__ hole_pix, uchar4* __restrict__ out) {
    const TapeHeader* h = reinterpret_cast<const TapeHeader*>(a.job0.tape);
    const uint32_t n = *count;
    V fog = ld3(h->fog);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float4 t4 = a.b.term[k];
        V v{t4.x, t4.y, t4.z};
        uint32_t lvl = __float_as_uint(t4.w);
        while (lvl > 0) {
            lvl -= 1;
            size_t li = ((size_t)lvl * a.cap + k) * 2;
            float4 A = a.b.lvl[li], B = a.b.lvl[li + 1];
            V r = scale(V{A.x, A.y, A.z}, 1.0f - A.w) + scale(v, A.w);
            r = r + V{B.x, B.y, B.z};
            v = apply_fog(r, fog, B.w, h->fog_density);
        }
        V d = display(v, h->exposure);
        out[hole_pix[k]] = make_uchar4(u8_of(d.x), u8_of(d.y), u8_of(d.z), 255);
    }
}

}  // namespace preview
}  // namespace mm3e
