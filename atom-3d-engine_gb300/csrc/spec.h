// spec.h — scene-specialised field programs compiled at run time with NVRTC.
//
// For a fixed scene the world field need not be interpreted: the generator emits CUDA source
// in which every object of the world plan is a call of the library's own object_field on a
// local constant copy of its tape record, and every segment of the plan is straight-line code
// that mirrors the interpreter's fold (ONE segments with the bounding-sphere substitute,
// LINEAR runs with the same prune / substitute / tie rules, big BVH runs and the rare LINEAR
// fallback through the shared bvh_segment walk). The compiler folds the constant records, so
// branches on flags and primitive kinds vanish and parameters become immediates, while every
// arithmetic operation stays the interpreter's, in its order: the specialised kernels give the
// interpreter's results bit for bit. The program instantiates the march / shadow / AO pass
// bodies of march_kernels.cuh with that field and is compiled for sm_103a straight to a cubin
// (no PTX is kept or read), loaded with cudaLibraryLoadData.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "kernels.h"

namespace mm3e {

// Source of the specialised program for a lowered tape blob (host copy).
std::string spec_source(const std::vector<unsigned char>& blob, uint32_t block, uint32_t unroll, bool smem_tape,
                        uint32_t min_blocks);

// Size of the generated field: objects it inlines and CSG program ops among them. Every inlined
// object is its own code (the interpreter shares one copy per primitive kind), so a large enough
// field outgrows the instruction cache. Measured with 64 field samples between refills: 1.3-2.6x
// faster than the interpreter on seeded scenes of 13 to 63 objects (1280x720).
struct SpecSize {
    uint32_t objects = 0, csg_ops = 0;
};
SpecSize spec_size(const std::vector<unsigned char>& blob);
// The automatic policy's limit.
constexpr uint32_t SPEC_AUTO_MAX_OBJECTS = 64;

// NVRTC compile of a specialised program to an sm_103a cubin (no device needed).
std::string spec_compile(const std::string& source, std::vector<char>& cubin);

class SpecModule {
  public:
    ~SpecModule();
    // Compiles `source` (NVRTC, sm_103a cubin) and loads its kernels. Returns "" or an error.
    std::string build(const std::string& source, int device, double* compile_ms);
    // Loads the kernels of a cubin spec_compile made (e.g. on another host thread).
    std::string load(const std::vector<char>& cubin, int device);
    SpecKernels kernels;

  private:
    cudaLibrary_t lib_ = nullptr;
};

// Whether NVRTC can be loaded in this process ("" when it can).
std::string nvrtc_status();

}  // namespace mm3e
