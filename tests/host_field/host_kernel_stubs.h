// Host stand-ins for the device-only builtins that march_kernels.cuh references, so that its
// per-lane march state machine (m_start / m_step) and the other kernels' bodies compile as plain
// C++ and a host loop can drive them item by item (tests/host_checks.py): one thread of one
// block, so a warp vote sees one lane and an atomic is a plain read-modify-write. Test
// infrastructure only.
#pragma once
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>
struct HostDim3 { unsigned x = 0, y = 0, z = 0; };
static thread_local HostDim3 threadIdx;  // per host thread, which plays one CUDA thread
static HostDim3 blockIdx, blockDim, gridDim;

// Barrier of the block host_launch is running (__syncthreads); none outside host_launch.
struct HostBlockBarrier {
    std::mutex m;
    std::condition_variable cv;
    unsigned n = 1, count = 0, gen = 0;
    void wait() {
        std::unique_lock<std::mutex> lock(m);
        const unsigned g = gen;
        if (++count == n) {
            count = 0;
            ++gen;
            cv.notify_all();
        } else {
            cv.wait(lock, [&] { return gen != g; });
        }
    }
};
static HostBlockBarrier* g_host_block_barrier = nullptr;
inline void __syncthreads() {
    if (g_host_block_barrier) g_host_block_barrier->wait();
}

// Runs `body` (a kernel call) as `grid` blocks of `block` host threads, one block at a time, so
// that a kernel's __shared__ storage (function-static on the host: define __shared__ as static
// before including it) and its __syncthreads() behave as on the device.
template <class F> void host_launch(unsigned grid, unsigned block, F body) {
    gridDim.x = grid;
    blockDim.x = block;
    HostBlockBarrier bar;
    bar.n = block;
    g_host_block_barrier = &bar;
    for (unsigned b = 0; b < grid; ++b) {
        blockIdx.x = b;
        std::vector<std::thread> threads;
        for (unsigned t = 0; t < block; ++t)
            threads.emplace_back([&body, t] {
                threadIdx.x = t;
                body();
            });
        for (auto& th : threads) th.join();
    }
    g_host_block_barrier = nullptr;
    gridDim.x = blockDim.x = 1;
    blockIdx.x = 0;
}
inline unsigned __ballot_sync(unsigned, int p) { return p ? 1u : 0u; }
template <class T> inline T __shfl_sync(unsigned, T v, int) { return v; }
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __ffs(int x) { return __builtin_ffs(x); }
inline unsigned atomicAdd(unsigned* p, unsigned v) { unsigned o = *p; *p += v; return o; }
inline size_t __cvta_generic_to_shared(const void*) { return 0; }
inline void __nanosleep(unsigned) {}
inline unsigned atomicOr(unsigned* p, unsigned v) { unsigned o = *p; *p |= v; return o; }
inline unsigned long long atomicMin(unsigned long long* p, unsigned long long v) {
    unsigned long long o = *p;
    if (v < o) *p = v;
    return o;
}
