// mesh.h — mesh -> signed-distance-grid bake on the GPU (mesh.rs bake_sdf).
//
// The host validates the mesh, sets up the grid (padded bounds, dims from the resolution along
// the longest axis) and builds the triangle BVH exactly as the reference does (median split of
// the longest centroid extent, ties by triangle index, one triangle per leaf), so the device's
// near-first nearest-triangle query visits nodes in the reference's order. One CTA per grid
// row (j, k) first collects the row's X-line crossings in shared memory (binary64 edge tests
// on binary32 vertices, the half-open ownership rule), then every thread samples grid points
// of the row: unsigned distance from the BVH query, negative where an odd number of
// crossings lies left of the point.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace mm3e {

// 32 bytes: bounds + children (inner) or -1 - triangle (leaf) in `a`.
struct alignas(16) DevTriNode {
    float lo[3];
    int32_t a;
    float hi[3];
    int32_t b;
};

struct MeshGrid {
    uint32_t nx = 0, ny = 0, nz = 0;
    float lo[3] = {0, 0, 0}, cell[3] = {0, 0, 0};
};

// Host side: validation, grid set-up and BVH (mesh.rs:30-52, 163-219, 266-283).
struct MeshPlan {
    MeshGrid grid;
    std::vector<float4> a, b, c;     // triangle vertices (xyz), all triangles in mesh order
    std::vector<float4> yz;          // per triangle: min y, max y, min z, max z
    std::vector<DevTriNode> nodes;   // BVH over the non-degenerate triangles
    uint32_t root = 0;
};
// Returns "" or the reference's error message.
std::string plan_mesh_bake(const float* positions, uint32_t n_positions, const uint32_t* triangles,
                           uint32_t n_triangles, uint32_t resolution, float padding, MeshPlan& out);

constexpr uint32_t MESH_ROW_CROSSINGS_MAX = 2048;
enum : uint32_t { ST_MESH_ROW_OVERFLOW = 4u, ST_MESH_STACK_OVERFLOW = 8u };

// Device side: all arrays on the device; data gets nx*ny*nz samples ((k*ny + j)*nx + i).
cudaError_t launch_mesh_bake(const MeshGrid& g, const float4* a, const float4* b, const float4* c, const float4* yz,
                             uint32_t n_tri, const DevTriNode* nodes, uint32_t root, float* data, uint32_t* status,
                             cudaStream_t s);

}  // namespace mm3e
