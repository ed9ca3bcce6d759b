// reproject.cu — launchers of the preview path's kernels (reproject_kernels.cuh): G-buffer
// packing and camera reprojection (mm3e-orchestrator/src/lib.rs:951-1080, reproject.rs:55-146).
#include <cuda_runtime.h>

#include "kernels.h"
#include "reproject_kernels.cuh"

namespace mm3e {
namespace {

using namespace preview;

unsigned grid_of(size_t n, uint32_t cap) {
    size_t g = (n + RP_THREADS - 1) / RP_THREADS;
    if (cap && g > cap) g = cap;
    return g ? (unsigned)g : 1u;
}

}  // namespace

cudaError_t launch_gbuffer_pack(const WaveArgs& a, uint32_t n_slots, const float4* movers, uint32_t n_movers,
                                uchar4* color, float* depth, int32_t* obj, cudaStream_t s, LaunchLog* log) {
    if (n_slots == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 1);
    k_gbuffer_pack<<<grid_of(n_slots, a.grid_cap), RP_THREADS, 0, s>>>(a, n_slots, movers, n_movers, color, depth, obj);
    return cudaGetLastError();
}

cudaError_t launch_warp(const CameraArgs& prev, const CameraArgs& next, uint32_t w, uint32_t h, const float* depth,
                        const int32_t* obj, const float* deltas3, uint32_t n_deltas, unsigned long long* keys,
                        const uchar4* src, uchar4* out, unsigned char* filled, cudaStream_t s, LaunchLog* log) {
    size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 2);
    cudaError_t e = cudaMemsetAsync(keys, 0xFF, n * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_warp_keys<<<grid_of(n, 0), RP_THREADS, 0, s>>>(prev, next, w, h, depth, obj, deltas3, n_deltas, keys);
    k_warp_apply<<<grid_of(n, 0), RP_THREADS, 0, s>>>((uint32_t)n, keys, src, out, filled);
    return cudaGetLastError();
}

cudaError_t launch_row_fill(uint32_t w, uint32_t h, uchar4* out, unsigned char* filled, cudaStream_t s,
                            LaunchLog* log) {
    if (w == 0 || h == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 1);
    k_row_fill<<<(h + 127) / 128, 128, 0, s>>>(w, h, out, filled);
    return cudaGetLastError();
}

cudaError_t launch_hole_rays(const CameraArgs& cam, uint32_t w, uint32_t h, const unsigned char* filled, float4* q_o,
                             float4* q_d, uint32_t* hole_pix, uint32_t* count, uint32_t grid_cap, cudaStream_t s,
                             LaunchLog* log) {
    size_t n = (size_t)w * h;
    if (n == 0) return cudaSuccess;
    LogScope sc(log, KK_OTHER, s, 1);
    k_hole_rays<<<grid_of(n, grid_cap), RP_THREADS, 0, s>>>(cam, w, h, filled, q_o, q_d, hole_pix, count);
    return cudaGetLastError();
}

cudaError_t launch_hole_resolve(const WaveArgs& a, const uint32_t* count, const uint32_t* hole_pix, uchar4* out,
                                cudaStream_t s, LaunchLog* log) {
    LogScope sc(log, KK_RESOLVE, s, 1);
    k_hole_resolve<<<grid_of(a.n_items, a.grid_cap), RP_THREADS, 0, s>>>(a, count, hole_pix, out);
    return cudaGetLastError();
}

}  // namespace mm3e
