// noalloc.h — allocation-free ray queries (scratch in a fixed __device__ array).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "kernels.h"

namespace mm3e {

constexpr size_t NOALLOC_MAX_RAYS = 262144;  // rays per call; scratch is about 14.7 MB per GPU

// March `n` device-resident rays (6 floats each) and write t / material (NIL on a miss) /
// steps into device buffers, using only the fixed scratch array, in the launch shape `tune`.
// `device` must be the current device. Blocking. Returns 0 on success, 1 for a size beyond
// NOALLOC_MAX_RAYS, 2 for a CUDA error, 3 for a tape-staging timeout; `what` receives a message.
int noalloc_march_rays(const unsigned char* tape, uint32_t tape_bytes, int device, int sm_count, cudaStream_t stream,
                       const TuneParams& tune, const float* d_rays6, size_t n, float* d_t, uint32_t* d_mat,
                       uint32_t* d_steps, const char** what);

}  // namespace mm3e
