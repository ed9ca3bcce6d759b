// lower.h — host-side validation and lowering of an mm3e_scene_desc into a scene tape.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mm3e_cuda.h"
#include "tape.h"

namespace mm3e {

// Result of lowering: the tape blob (header + sections) plus the places where device
// addresses of large payloads must be patched in after upload.
struct LoweredScene {
    std::vector<unsigned char> blob;  // 16-byte aligned sections, header first
    uint32_t width = 0, height = 0, mode = 0, aa = 1, bounces = 0;
    bool dual_safe = false;
    bool has_gi = false;
    uint32_t bvh_depth = 0;           // deepest BVH (levels)
    uint32_t csg_stack = 0;           // deepest CSG value/point stack
    // payloads to upload (volume samples, GI cubes) and their patch offsets in the blob
    struct Payload {
        const void* host;
        size_t bytes;
        size_t patch_offset;  // byte offset of the `const T*` field inside blob
    };
    std::vector<Payload> payloads;
    std::vector<float> gi_float4;     // GI cubes converted to float4 per face
};

// Validates `d` (reference rules plus this path's limits). Returns MM3E_OK or an error code
// with a message.
int validate_scene(const mm3e_scene_desc& d, std::string& err);

// Validates dynamic spheres exactly as CpuParallelScene::try_render (mm3e-cpu-parallel
// src/lib.rs:55-57, 68-84).
int validate_dynamic(const mm3e_scene_desc& d, const mm3e_dyn_sphere* dyn, size_t n, std::string& err);

// Lowers a validated scene. `dyn`/`n_dyn` append dynamic spheres as real objects and
// materials (Union, Material::default() fields otherwise), as try_render does.
int lower_scene(const mm3e_scene_desc& d, const mm3e_dyn_sphere* dyn, size_t n_dyn, LoweredScene& out,
                std::string& err);

// Normalised Gaussian bloom weights of radius max(radius, 1): 2r + 1 taps (post.rs:331-345).
std::vector<float> gaussian_kernel(uint32_t radius);

// GI bake set-up (Scene::bake_gi_unchecked, lib.rs:668-682; gi.rs:38-72,192-203): probe grid
// bounds from the objects' world bounding spheres padded by 1.5, the cell size, and the
// per-face gather directions with their weights (axis first, then four 45-degree tilts).
struct GiSetup {
    float lo[3], size[3], cell[3];
    uint32_t nx, ny, nz, dirs_per_face;
    std::vector<float> dirs;  // 6 faces x dirs_per_face x (x, y, z, weight)
};
// Returns false when no object has a finite bound (the reference then leaves GI unchanged).
bool gi_setup(const mm3e_scene_desc& d, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t samples, GiSetup& out);

}  // namespace mm3e
