// Host stand-ins for the device-only builtins that march_kernels.cuh references, so that its
// per-lane march state machine (m_start / m_step) and the other kernels' bodies compile as plain
// C++ and a host loop can drive them item by item (tests/test_spec_host_cpu.py): one thread of one
// block, so a warp vote sees one lane and an atomic is a plain read-modify-write. Test
// infrastructure only.
#pragma once
struct HostDim3 { unsigned x = 0, y = 0, z = 0; };
static HostDim3 threadIdx, blockIdx, blockDim, gridDim;
inline void __syncthreads() {}
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
