// mesh_bake.cu — sm_103a kernel of the mesh -> SDF bake (mesh.rs:106-146, 221-336;
// triangle.rs:4-34). One CTA per grid row; binary32 arithmetic without contraction (the
// library is compiled with --fmad=false) and binary64 crossing tests, as the reference.
#include <cuda_runtime.h>

#include "mesh.h"

namespace mm3e {
namespace {

constexpr int ROW_THREADS = 128;
constexpr int STACK = 64;  // the reference's fixed traversal stack

struct P3 {
    float x, y, z;
};
__device__ __forceinline__ P3 sub(P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ P3 add(P3 a, P3 b) { return P3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ P3 scl(P3 a, float s) { return P3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot3(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ P3 ld(float4 v) { return P3{v.x, v.y, v.z}; }

// closest_on_triangle (mesh.rs:106-146)
__device__ __forceinline__ P3 closest_on_triangle(P3 p, P3 a, P3 b, P3 c) {
    P3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    P3 bp = sub(p, b);
    float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return add(a, scl(ab, d1 / (d1 - d3)));
    P3 cp = sub(p, c);
    float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return add(a, scl(ac, d2 / (d2 - d6)));
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return add(b, scl(sub(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6))));
    float denom = 1.0f / (va + vb + vc);
    return add(add(a, scl(ab, vb * denom)), scl(ac, vc * denom));
}

__device__ __forceinline__ float box_dist_sq(P3 p, const DevTriNode& n) {
    P3 q{fminf(fmaxf(p.x, n.lo[0]), n.hi[0]), fminf(fmaxf(p.y, n.lo[1]), n.hi[1]), fminf(fmaxf(p.z, n.lo[2]), n.hi[2])};
    P3 d = sub(p, q);
    return dot3(d, d);
}

// triangle.rs:4-34
__device__ __forceinline__ double edge(P3 a, P3 b, double y, double z) {
    return ((double)b.y - (double)a.y) * (z - (double)a.z) - ((double)b.z - (double)a.z) * (y - (double)a.y);
}
__device__ __forceinline__ bool owns_boundary(P3 a, P3 b) { return b.z > a.z || (b.z == a.z && b.y < a.y); }
__device__ __forceinline__ bool x_crossing(P3 a, P3 b, P3 c, float yf, float zf, float& out) {
    double area = edge(a, b, (double)c.y, (double)c.z);
    if (area == 0.0 || !isfinite(area) || !isfinite(yf) || !isfinite(zf)) return false;
    if (area < 0.0) {
        P3 t = b;
        b = c;
        c = t;
        area = -area;
    }
    double y = yf, z = zf;
    double w0 = edge(b, c, y, z), w1 = edge(c, a, y, z), w2 = edge(a, b, y, z);
    if (w0 < 0.0 || (w0 == 0.0 && !owns_boundary(b, c))) return false;
    if (w1 < 0.0 || (w1 == 0.0 && !owns_boundary(c, a))) return false;
    if (w2 < 0.0 || (w2 == 0.0 && !owns_boundary(a, b))) return false;
    float x = (float)((w0 * (double)a.x + w1 * (double)b.x + w2 * (double)c.x) / area);
    if (!isfinite(x)) return false;
    out = x;
    return true;
}

// TriBvh::nearest_sq (mesh.rs:221-254): same node order as the reference.
__device__ float nearest_sq(const DevTriNode* __restrict__ nodes, uint32_t root, const float4* __restrict__ A,
                            const float4* __restrict__ B, const float4* __restrict__ C, P3 p, bool& overflow) {
    float best = __int_as_float(0x7f800000);
    uint32_t stack[STACK];
    int sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const DevTriNode n = nodes[stack[--sp]];
        if (box_dist_sq(p, n) >= best) continue;
        if (n.a < 0) {
            uint32_t t = (uint32_t)(-1 - n.a);
            P3 q = closest_on_triangle(p, ld(A[t]), ld(B[t]), ld(C[t]));
            P3 d = sub(p, q);
            best = fminf(best, dot3(d, d));
        } else {
            uint32_t l = (uint32_t)n.a, r = (uint32_t)n.b;
            float ldist = box_dist_sq(p, nodes[l]);
            float rdist = box_dist_sq(p, nodes[r]);
            if (sp + 2 > STACK) {
                overflow = true;
                return __int_as_float(0x7fc00000);
            }
            stack[sp] = ldist <= rdist ? r : l;
            stack[sp + 1] = ldist <= rdist ? l : r;
            sp += 2;
        }
    }
    return best;
}

__global__ void __launch_bounds__(ROW_THREADS)
    k_mesh_rows(MeshGrid g, const float4* __restrict__ A, const float4* __restrict__ B, const float4* __restrict__ C,
                const float4* __restrict__ YZ, uint32_t n_tri, const DevTriNode* __restrict__ nodes, uint32_t root,
                float* __restrict__ data, uint32_t* status) {
    __shared__ float xs[MESH_ROW_CROSSINGS_MAX];
    __shared__ uint32_t nx_cross;
    __shared__ uint32_t overflow;
    const uint32_t row = blockIdx.x;  // k * ny + j
    const uint32_t j = row % g.ny, k = row / g.ny;
    const float y = g.lo[1] + (float)j * g.cell[1];
    const float z = g.lo[2] + (float)k * g.cell[2];
    if (threadIdx.x == 0) {
        nx_cross = 0;
        overflow = 0;
    }
    __syncthreads();
    // row crossings: only triangles whose YZ bounds hold (y, z) can be crossed (the binary64
    // edge tests are exact in sign, so the bound test never drops a crossing)
    for (uint32_t t = threadIdx.x; t < n_tri; t += ROW_THREADS) {
        float4 bb = YZ[t];
        if (y < bb.x || y > bb.y || z < bb.z || z > bb.w) continue;
        float x;
        if (x_crossing(ld(A[t]), ld(B[t]), ld(C[t]), y, z, x)) {
            uint32_t slot = atomicAdd(&nx_cross, 1u);
            if (slot < MESH_ROW_CROSSINGS_MAX) xs[slot] = x;
            else overflow = 1u;
        }
    }
    __syncthreads();
    if (overflow) {
        if (threadIdx.x == 0) atomicOr(status, ST_MESH_ROW_OVERFLOW);
        return;
    }
    const uint32_t nc = nx_cross;
    bool stack_overflow = false;
    for (uint32_t i = threadIdx.x; i < g.nx; i += ROW_THREADS) {
        P3 p{g.lo[0] + (float)i * g.cell[0], y, z};
        float u = sqrtf(nearest_sq(nodes, root, A, B, C, p, stack_overflow));
        uint32_t left = 0;
        for (uint32_t c = 0; c < nc; ++c) left += xs[c] < p.x ? 1u : 0u;
        data[((size_t)k * g.ny + j) * g.nx + i] = (left & 1u) ? -u : u;
    }
    if (stack_overflow) atomicOr(status, ST_MESH_STACK_OVERFLOW);
}

}  // namespace

cudaError_t launch_mesh_bake(const MeshGrid& g, const float4* a, const float4* b, const float4* c, const float4* yz,
                             uint32_t n_tri, const DevTriNode* nodes, uint32_t root, float* data, uint32_t* status,
                             cudaStream_t s) {
    uint64_t rows = (uint64_t)g.ny * g.nz;
    if (rows == 0 || g.nx == 0) return cudaSuccess;
    k_mesh_rows<<<(unsigned)rows, ROW_THREADS, 0, s>>>(g, a, b, c, yz, n_tri, nodes, root, data, status);
    return cudaGetLastError();
}

}  // namespace mm3e
