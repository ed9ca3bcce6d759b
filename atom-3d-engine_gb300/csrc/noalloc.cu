// noalloc.cu — allocation-free ray queries (mm3e_march_rays_noalloc).
//
// Some callers cannot allocate device memory at query time: a game or simulation loop that
// issues picking / collision rays every frame cannot afford cudaMalloc or cudaFree (both
// synchronise the device and can stall for milliseconds), and a service whose device memory
// was fully reserved up front (a fixed pool or an admission budget) has nothing left to
// allocate from. For them the march kernel's scratch — the ray queue and the hit records —
// lives in one file-scope __device__ array of fixed size, so a query allocates nothing: the
// caller passes device input and output buffers and the library only launches kernels.
//
// The array is shared by every call on a device and keeps the previous call's contents; the
// work counters are cleared at the start of each call. Calls that overlap on the GPU (from
// different host threads or streams) race on the array and must be serialised by the caller.
// Each GPU that loads the library holds the array (about 14.7 MB) until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.h"
#include "noalloc.h"

namespace mm3e {
namespace {

struct NoAllocScratch {
    float4 q_o[NOALLOC_MAX_RAYS];
    float4 q_d[NOALLOC_MAX_RAYS];
    float4 h_n[NOALLOC_MAX_RAYS];
    uint2 h_m[NOALLOC_MAX_RAYS];
    uint32_t counters[64];  // [0] work counter, [63] status word
};

static __device__ __align__(256) NoAllocScratch g_noalloc;

// Device address of g_noalloc per device (host code cannot use the symbol's name as an address).
constexpr int MAX_DEVICES = 64;
NoAllocScratch* g_addr[MAX_DEVICES] = {};
std::mutex g_mu;

__global__ void k_pack_rays(const float* __restrict__ rays6, uint32_t n, float4* __restrict__ o,
                            float4* __restrict__ d) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays6 + 6 * (size_t)i;
    o[i] = make_float4(r[0], r[1], r[2], 0.0f);
    d[i] = make_float4(r[3], r[4], r[5], 0.0f);
}

__global__ void k_split_hits(const float4* __restrict__ hn, const uint2* __restrict__ hm, uint32_t n,
                             float* __restrict__ t, uint32_t* __restrict__ mat, uint32_t* __restrict__ steps) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    t[i] = hn[i].w;
    uint2 m = hm[i];
    mat[i] = m.x;
    if (steps) steps[i] = m.y;
}

// Set-up, once per device, with that device current: resolve the array's device address. The
// address is cached for the life of the process's context on that device; cudaDeviceReset
// ends that context (and every scene and stream of this library on it) and invalidates it.
cudaError_t scratch_for(int device, NoAllocScratch** out) {
    if (device < 0 || device >= MAX_DEVICES) return cudaErrorInvalidDevice;
    int current = -1;
    cudaError_t ce = cudaGetDevice(&current);
    if (ce != cudaSuccess) return ce;
    if (current != device) return cudaErrorInvalidDevice;  // the address is per device
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc);
        if (e != cudaSuccess) return e;
        g_addr[device] = static_cast<NoAllocScratch*>(p);
    }
    *out = g_addr[device];
    return cudaSuccess;
}

}  // namespace

int noalloc_march_rays(const unsigned char* tape, uint32_t tape_bytes, int device, int sm_count, cudaStream_t stream,
                       const TuneParams& tune, const float* d_rays6, size_t n, float* d_t, uint32_t* d_mat,
                       uint32_t* d_steps, const char** what) {
    *what = "";
    if (n == 0) return 0;
    if (n > NOALLOC_MAX_RAYS) {
        *what = "mm3e_march_rays_noalloc takes at most 262144 rays per call";
        return 1;
    }
    NoAllocScratch* s = nullptr;
    cudaError_t e = scratch_for(device, &s);
    if (e != cudaSuccess) {
        *what = cudaGetErrorString(e);
        return 2;
    }
    uint32_t nn = (uint32_t)n;
    unsigned blocks = (nn + 127) / 128;
    e = cudaMemsetAsync(s->counters, 0, sizeof(s->counters), stream);
    if (e == cudaSuccess) {
        k_pack_rays<<<blocks, 128, 0, stream>>>(d_rays6, nn, s->q_o, s->q_d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        WaveArgs a{};
        a.job0.tape = tape;
        a.tape_bytes = tape_bytes;
        a.status = s->counters + 63;
        a.counter = s->counters;
        a.src = SRC_QUEUE;
        a.n_items = nn;
        a.cap = nn;
        a.b.q_o = s->q_o;
        a.b.q_d = s->q_d;
        a.b.h_n = s->h_n;
        a.b.h_m = s->h_m;
        e = launch_march(a, tune, stream, sm_count, nullptr);
    }
    if (e == cudaSuccess) {
        k_split_hits<<<blocks, 128, 0, stream>>>(s->h_n, s->h_m, nn, d_t, d_mat, d_steps);
        e = cudaGetLastError();
    }
    uint32_t status = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, s->counters + 63, sizeof(status), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        *what = cudaGetErrorString(e);
        return 2;
    }
    if (status & ST_TAPE_TIMEOUT) {
        *what = "scene tape staging wait gave up";
        return 3;
    }
    if (status) {
        *what = "scene tape corrupt after staging";
        return 2;
    }
    return 0;
}

}  // namespace mm3e
