// mesh.cpp — host half of the mesh -> SDF bake: validation, grid set-up, the triangle BVH
// (mesh.rs:30-52, 163-219, 266-283) and the C ABI entry mm3e_bake_mesh_sdf. Binary32 host
// arithmetic without contraction (compiled with -ffp-contract=off), min/max ignoring NaN as
// Rust's f32::min / f32::max.
#include "mesh.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "capi_internal.h"

namespace mm3e {
namespace {

struct H3 {
    float x, y, z;
};
H3 operator-(H3 a, H3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
H3 operator+(H3 a, H3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
H3 hmin(H3 a, H3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
H3 hmax(H3 a, H3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
H3 hscale(H3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float hlen_sq(H3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
H3 hcross(H3 a, H3 o) { return {a.y * o.z - a.z * o.y, a.z * o.x - a.x * o.z, a.x * o.y - a.y * o.x}; }

struct BuildItem {
    uint32_t idx;
    H3 lo, hi, c;
};

// Children are emitted before their parent, as the reference's recursive build does.
int32_t build_node(BuildItem* items, size_t n, std::vector<DevTriNode>& nodes) {
    H3 lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < n; ++i) {
        lo = hmin(lo, items[i].lo);
        hi = hmax(hi, items[i].hi);
    }
    DevTriNode node{};
    node.lo[0] = lo.x;
    node.lo[1] = lo.y;
    node.lo[2] = lo.z;
    node.hi[0] = hi.x;
    node.hi[1] = hi.y;
    node.hi[2] = hi.z;
    if (n == 1) {
        node.a = -1 - (int32_t)items[0].idx;
        node.b = 0;
        nodes.push_back(node);
        return (int32_t)nodes.size() - 1;
    }
    H3 clo{INFINITY, INFINITY, INFINITY}, chi{-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < n; ++i) {
        clo = hmin(clo, items[i].c);
        chi = hmax(chi, items[i].c);
    }
    H3 ext = chi - clo;
    int axis = (ext.x >= ext.y && ext.x >= ext.z) ? 0 : (ext.y >= ext.z ? 1 : 2);
    auto key = [axis](const BuildItem& it) { return axis == 0 ? it.c.x : axis == 1 ? it.c.y : it.c.z; };
    std::sort(items, items + n, [&](const BuildItem& p, const BuildItem& q) {
        float kp = key(p), kq = key(q);
        if (kp < kq) return true;
        if (kq < kp) return false;
        return p.idx < q.idx;
    });
    size_t mid = n / 2;
    int32_t left = build_node(items, mid, nodes);
    int32_t right = build_node(items + mid, n - mid, nodes);
    node.a = left;
    node.b = right;
    nodes.push_back(node);
    return (int32_t)nodes.size() - 1;
}

}  // namespace

std::string plan_mesh_bake(const float* positions, uint32_t n_positions, const uint32_t* triangles,
                           uint32_t n_triangles, uint32_t resolution, float padding, MeshPlan& out) {
    // Mesh::validate (mesh.rs:30-52)
    if (n_positions == 0 || !positions) return "mesh has no vertices";
    if (n_triangles == 0 || !triangles) return "mesh has no triangles";
    std::vector<H3> pos(n_positions);
    for (uint32_t i = 0; i < n_positions; ++i) {
        pos[i] = H3{positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]};
        if (!std::isfinite(pos[i].x) || !std::isfinite(pos[i].y) || !std::isfinite(pos[i].z))
            return "mesh vertex " + std::to_string(i) + " is non-finite";
    }
    for (uint32_t t = 0; t < n_triangles; ++t)
        for (int k = 0; k < 3; ++k)
            if (triangles[3 * t + k] >= n_positions)
                return "mesh triangle " + std::to_string(t) + " references a vertex out of range";
    // bake_sdf grid (mesh.rs:266-283)
    H3 mlo{INFINITY, INFINITY, INFINITY}, mhi{-INFINITY, -INFINITY, -INFINITY};
    for (const H3& p : pos) {
        mlo = hmin(mlo, p);
        mhi = hmax(mhi, p);
    }
    if (!(padding > 0.0f) || !std::isfinite(padding)) return "padding must be positive and finite";
    uint32_t res = std::min<uint32_t>(std::max<uint32_t>(resolution, 2u), 512u);
    H3 lo = mlo - H3{padding, padding, padding}, hi = mhi + H3{padding, padding, padding};
    H3 size = hi - lo;
    float longest = std::fmax(std::fmax(std::fmax(size.x, size.y), size.z), 1e-6f);
    auto dim = [&](float s) {
        float v = std::round((s / longest) * (float)(res - 1));
        uint64_t d = (uint64_t)(v > 0.0f ? v : 0.0f) + 1;
        return (uint32_t)std::max<uint64_t>(d, 2);
    };
    MeshGrid& g = out.grid;
    g.nx = dim(size.x);
    g.ny = dim(size.y);
    g.nz = dim(size.z);
    g.lo[0] = lo.x;
    g.lo[1] = lo.y;
    g.lo[2] = lo.z;
    g.cell[0] = size.x / (float)(g.nx - 1);
    g.cell[1] = size.y / (float)(g.ny - 1);
    g.cell[2] = size.z / (float)(g.nz - 1);
    // triangle arrays and the BVH (mesh.rs:198-219)
    out.a.resize(n_triangles);
    out.b.resize(n_triangles);
    out.c.resize(n_triangles);
    out.yz.resize(n_triangles);
    std::vector<BuildItem> items;
    items.reserve(n_triangles);
    for (uint32_t t = 0; t < n_triangles; ++t) {
        H3 a = pos[triangles[3 * t]], b = pos[triangles[3 * t + 1]], c = pos[triangles[3 * t + 2]];
        out.a[t] = make_float4(a.x, a.y, a.z, 0.0f);
        out.b[t] = make_float4(b.x, b.y, b.z, 0.0f);
        out.c[t] = make_float4(c.x, c.y, c.z, 0.0f);
        out.yz[t] = make_float4(std::fmin(std::fmin(a.y, b.y), c.y), std::fmax(std::fmax(a.y, b.y), c.y),
                                std::fmin(std::fmin(a.z, b.z), c.z), std::fmax(std::fmax(a.z, b.z), c.z));
        if (hlen_sq(hcross(b - a, c - a)) < 1e-16f) continue;
        items.push_back(BuildItem{t, hmin(hmin(a, b), c), hmax(hmax(a, b), c), hscale((a + b) + c, 1.0f / 3.0f)});
    }
    if (items.empty()) return "mesh has no non-degenerate triangles";
    out.nodes.clear();
    out.nodes.reserve(items.size() * 2);
    out.root = (uint32_t)build_node(items.data(), items.size(), out.nodes);
    return "";
}

}  // namespace mm3e

using namespace mm3e;

extern "C" {

int mm3e_bake_mesh_sdf(mm3e_ctx* ctx, const mm3e_mesh* mesh, uint32_t resolution, float padding, mm3e_volume* out,
                       float* data, size_t n_floats, int data_on_device) {
    if (!ctx || !mesh || !out) return MM3E_ERR_INVALID;
    MeshPlan plan;
    std::string err = plan_mesh_bake(mesh->positions, mesh->n_positions, mesh->triangles, mesh->n_triangles, resolution,
                                     padding, plan);
    if (!err.empty()) return fail(ctx, MM3E_ERR_INVALID, err);
    const MeshGrid& g = plan.grid;
    out->nx = g.nx;
    out->ny = g.ny;
    out->nz = g.nz;
    std::memcpy(out->min, g.lo, 12);
    std::memcpy(out->cell, g.cell, 12);
    out->data = nullptr;
    size_t n = (size_t)g.nx * g.ny * g.nz;
    if (!data) return MM3E_OK;  // grid query only
    if (n_floats < n) return fail(ctx, MM3E_ERR_INVALID, "volume buffer too small");
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    uint32_t nt = mesh->n_triangles;
    float4 *d_a = nullptr, *d_b = nullptr, *d_c = nullptr, *d_yz = nullptr;
    DevTriNode* d_nodes = nullptr;
    float* d_data = data_on_device ? data : nullptr;
    uint32_t* d_status = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d_a), nt * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_b), nt * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_c), nt * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_yz), nt * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_nodes), plan.nodes.size() * sizeof(DevTriNode));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_status), sizeof(uint32_t));
    if (e == cudaSuccess && !data_on_device) e = cudaMalloc(reinterpret_cast<void**>(&d_data), n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_a, plan.a.data(), nt * sizeof(float4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_b, plan.b.data(), nt * sizeof(float4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_c, plan.c.data(), nt * sizeof(float4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_yz, plan.yz.data(), nt * sizeof(float4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_nodes, plan.nodes.data(), plan.nodes.size() * sizeof(DevTriNode), cudaMemcpyHostToDevice,
                            s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(uint32_t), s);
    LaunchLog log = ctx->prof.log();
    if (e == cudaSuccess) {
        if (log.begin) log.begin(log.recorder, KK_OTHER, s);
        e = launch_mesh_bake(g, d_a, d_b, d_c, d_yz, nt, d_nodes, plan.root, d_data, d_status, s);
        if (log.end) log.end(log.recorder, KK_OTHER, s);
    }
    uint32_t status = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && !data_on_device) e = cudaMemcpyAsync(data, d_data, n * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_a);
    cudaFree(d_b);
    cudaFree(d_c);
    cudaFree(d_yz);
    cudaFree(d_nodes);
    cudaFree(d_status);
    if (!data_on_device) cudaFree(d_data);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mesh bake");
    if (status & ST_MESH_ROW_OVERFLOW)
        return fail(ctx, MM3E_ERR_UNSUPPORTED,
                    "a grid row crosses more than " + std::to_string(MESH_ROW_CROSSINGS_MAX) + " triangles");
    if (status & ST_MESH_STACK_OVERFLOW) return fail(ctx, MM3E_ERR_UNSUPPORTED, "triangle BVH deeper than 64 levels");
    if (!data_on_device) out->data = data;
    return MM3E_OK;
}

}  // extern "C"
