// oracle_mesh.hpp — CPU restatement of the reference's mesh -> SDF bake.
//
// TEST INFRASTRUCTURE ONLY: the checker the CUDA mesh bake is compared against, never a
// product path. Follows mm3e-orchestrator/src/mesh.rs:106-336 (closest point on a triangle,
// the triangle BVH with its median split and near-first nearest query, bake_sdf's grid set-up
// and row-parity sign) and mm3e-kit/src/triangle.rs:4-34 (x_crossing in binary64 on binary32
// inputs, half-open edge ownership). Binary32 arithmetic is done as Rust does it: no
// contraction (this code is compiled with -ffp-contract=off), min/max ignore NaN.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <thread>
#include <vector>

namespace oracle {
namespace mesh {

struct F3 {
    float x, y, z;
};
inline F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 scale(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline F3 cross(F3 a, F3 o) { return {a.y * o.z - a.z * o.y, a.z * o.x - a.x * o.z, a.x * o.y - a.y * o.x}; }
inline float length_sq(F3 a) { return dot(a, a); }
inline F3 vmin(F3 a, F3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline F3 vmax(F3 a, F3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
inline F3 splat(float v) { return {v, v, v}; }

// mesh.rs:106-146
inline F3 closest_on_triangle(F3 p, F3 a, F3 b, F3 c) {
    F3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    F3 bp = p - b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return a + scale(ab, d1 / (d1 - d3));
    F3 cp = p - c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return a + scale(ac, d2 / (d2 - d6));
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return b + scale(c - b, (d4 - d3) / ((d4 - d3) + (d5 - d6)));
    float denom = 1.0f / (va + vb + vc);
    return a + scale(ab, vb * denom) + scale(ac, vc * denom);
}

// triangle.rs:4-34
inline double edge(F3 a, F3 b, double y, double z) {
    return ((double)b.y - (double)a.y) * (z - (double)a.z) - ((double)b.z - (double)a.z) * (y - (double)a.y);
}
inline bool owns_boundary(F3 a, F3 b) { return b.z > a.z || (b.z == a.z && b.y < a.y); }
inline bool x_crossing(F3 a, F3 b, F3 c, float yf, float zf, float& out) {
    double area = edge(a, b, (double)c.y, (double)c.z);
    if (area == 0.0 || !std::isfinite(area) || !std::isfinite(yf) || !std::isfinite(zf)) return false;
    if (area < 0.0) {
        std::swap(b, c);
        area = -area;
    }
    double y = yf, z = zf;
    double w[3] = {edge(b, c, y, z), edge(c, a, y, z), edge(a, b, y, z)};
    F3 st[3] = {b, c, a}, en[3] = {c, a, b};
    for (int i = 0; i < 3; ++i)
        if (w[i] < 0.0 || (w[i] == 0.0 && !owns_boundary(st[i], en[i]))) return false;
    float x = (float)((w[0] * (double)a.x + w[1] * (double)b.x + w[2] * (double)c.x) / area);
    if (!std::isfinite(x)) return false;
    out = x;
    return true;
}

struct Mesh {
    std::vector<F3> pos;
    std::vector<uint32_t> tri;  // 3 per triangle
    F3 v(uint32_t t, int k) const { return pos[tri[3 * t + k]]; }
    size_t n_tri() const { return tri.size() / 3; }
};

struct TriNode {
    F3 lo, hi;
    uint32_t left, right;
    int32_t leaf;
};

struct Item {
    uint32_t idx;
    F3 lo, hi, c;
};

// TriBvh::build_from (mesh.rs:163-196): median split of the longest centroid extent, items
// ordered by that coordinate then index; one triangle per leaf; children before parents.
inline uint32_t build_from(Item* items, size_t n, std::vector<TriNode>& nodes) {
    F3 lo = splat(INFINITY), hi = splat(-INFINITY);
    for (size_t i = 0; i < n; ++i) {
        lo = vmin(lo, items[i].lo);
        hi = vmax(hi, items[i].hi);
    }
    if (n == 1) {
        nodes.push_back(TriNode{lo, hi, 0, 0, (int32_t)items[0].idx});
        return (uint32_t)(nodes.size() - 1);
    }
    F3 clo = splat(INFINITY), chi = splat(-INFINITY);
    for (size_t i = 0; i < n; ++i) {
        clo = vmin(clo, items[i].c);
        chi = vmax(chi, items[i].c);
    }
    F3 ext = chi - clo;
    int axis = (ext.x >= ext.y && ext.x >= ext.z) ? 0 : (ext.y >= ext.z ? 1 : 2);
    auto coord = [axis](const Item& it) { return axis == 0 ? it.c.x : axis == 1 ? it.c.y : it.c.z; };
    std::sort(items, items + n, [&](const Item& a, const Item& b) {
        float ca = coord(a), cb = coord(b);
        if (ca < cb) return true;
        if (cb < ca) return false;
        return a.idx < b.idx;  // partial_cmp Equal (or NaN) then index
    });
    size_t mid = n / 2;
    uint32_t left = build_from(items, mid, nodes);
    uint32_t right = build_from(items + mid, n - mid, nodes);
    nodes.push_back(TriNode{lo, hi, left, right, -1});
    return (uint32_t)(nodes.size() - 1);
}

// TriBvh::build (mesh.rs:198-219): degenerate triangles (|cross|^2 < 1e-16) are left out.
inline bool build_bvh(const Mesh& m, std::vector<TriNode>& nodes, uint32_t& root) {
    std::vector<Item> items;
    for (uint32_t t = 0; t < m.n_tri(); ++t) {
        F3 a = m.v(t, 0), b = m.v(t, 1), c = m.v(t, 2);
        if (length_sq(cross(b - a, c - a)) < 1e-16f) continue;
        items.push_back(Item{t, vmin(vmin(a, b), c), vmax(vmax(a, b), c), scale((a + b) + c, 1.0f / 3.0f)});
    }
    if (items.empty()) return false;
    nodes.clear();
    nodes.reserve(items.size() * 2);
    root = build_from(items.data(), items.size(), nodes);
    return true;
}

inline float box_dist_sq(F3 p, F3 lo, F3 hi) { return length_sq(p - vmin(vmax(p, lo), hi)); }

// TriBvh::nearest_sq (mesh.rs:221-254)
inline float nearest_sq(const std::vector<TriNode>& nodes, uint32_t root, F3 p, const Mesh& m) {
    float best = INFINITY;
    uint32_t stack[64];
    size_t sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const TriNode& node = nodes[stack[--sp]];
        if (box_dist_sq(p, node.lo, node.hi) >= best) continue;
        if (node.leaf >= 0) {
            uint32_t t = (uint32_t)node.leaf;
            F3 q = closest_on_triangle(p, m.v(t, 0), m.v(t, 1), m.v(t, 2));
            best = std::fmin(best, length_sq(p - q));
        } else {
            uint32_t l = node.left, r = node.right;
            float ld = box_dist_sq(p, nodes[l].lo, nodes[l].hi);
            float rd = box_dist_sq(p, nodes[r].lo, nodes[r].hi);
            uint32_t nr = ld <= rd ? l : r, fr = ld <= rd ? r : l;
            if (sp + 2 > 64) return NAN;  // deeper than the reference's fixed stack
            stack[sp] = fr;
            stack[sp + 1] = nr;
            sp += 2;
        }
    }
    return best;
}

struct Grid {
    uint32_t nx, ny, nz;
    F3 lo, cell;
};

// bake_sdf grid set-up (mesh.rs:266-283). Returns an error message or "".
inline std::string bake_grid(const Mesh& m, uint32_t resolution, float padding, Grid& g) {
    if (m.pos.empty()) return "mesh has no vertices";
    if (m.tri.empty()) return "mesh has no triangles";
    for (size_t i = 0; i < m.pos.size(); ++i)
        if (!std::isfinite(m.pos[i].x) || !std::isfinite(m.pos[i].y) || !std::isfinite(m.pos[i].z))
            return "mesh vertex " + std::to_string(i) + " is non-finite";
    for (size_t t = 0; t < m.n_tri(); ++t)
        for (int k = 0; k < 3; ++k)
            if (m.tri[3 * t + k] >= m.pos.size())
                return "mesh triangle " + std::to_string(t) + " references a vertex out of range";
    F3 mlo = splat(INFINITY), mhi = splat(-INFINITY);
    for (const F3& p : m.pos) {
        mlo = vmin(mlo, p);
        mhi = vmax(mhi, p);
    }
    if (!(padding > 0.0f) || !std::isfinite(padding)) return "padding must be positive and finite";
    uint32_t res = std::min<uint32_t>(std::max<uint32_t>(resolution, 2u), 512u);
    F3 lo = mlo - splat(padding), hi = mhi + splat(padding);
    F3 size = hi - lo;
    float longest = std::fmax(std::fmax(std::fmax(size.x, size.y), size.z), 1e-6f);
    auto dim = [&](float s) {
        float v = std::round((s / longest) * (float)(res - 1));
        uint64_t d = (uint64_t)(v > 0.0f ? v : 0.0f) + 1;
        return (uint32_t)std::max<uint64_t>(d, 2);
    };
    g.nx = dim(size.x);
    g.ny = dim(size.y);
    g.nz = dim(size.z);
    g.lo = lo;
    g.cell = F3{size.x / (float)(g.nx - 1), size.y / (float)(g.ny - 1), size.z / (float)(g.nz - 1)};
    return "";
}

// bake_sdf samples (mesh.rs:284-335): unsigned nearest distance, negated where the row's
// crossings left of the sample are odd. data: nx*ny*nz, (k*ny + j)*nx + i.
inline std::string bake_sdf(const Mesh& m, uint32_t resolution, float padding, Grid& g, std::vector<float>& data,
                            unsigned threads = 1) {
    std::string err = bake_grid(m, resolution, padding, g);
    if (!err.empty()) return err;
    std::vector<TriNode> nodes;
    uint32_t root = 0;
    if (!build_bvh(m, nodes, root)) return "mesh has no non-degenerate triangles";
    data.assign((size_t)g.nx * g.ny * g.nz, 0.0f);
    auto slab = [&](uint32_t k0, uint32_t k1) {
        std::vector<float> xs;
        for (uint32_t k = k0; k < k1; ++k) {
            float z = g.lo.z + (float)k * g.cell.z;
            for (uint32_t j = 0; j < g.ny; ++j) {
                float y = g.lo.y + (float)j * g.cell.y;
                xs.clear();
                for (uint32_t t = 0; t < m.n_tri(); ++t) {
                    float x;
                    if (x_crossing(m.v(t, 0), m.v(t, 1), m.v(t, 2), y, z, x)) xs.push_back(x);
                }
                std::sort(xs.begin(), xs.end());
                for (uint32_t i = 0; i < g.nx; ++i) {
                    F3 p{g.lo.x + (float)i * g.cell.x, g.lo.y + (float)j * g.cell.y, g.lo.z + (float)k * g.cell.z};
                    float unsigned_d = std::sqrt(nearest_sq(nodes, root, p, m));
                    size_t left = (size_t)(std::lower_bound(xs.begin(), xs.end(), p.x) - xs.begin());
                    bool inside = left % 2 == 1;
                    data[((size_t)k * g.ny + j) * g.nx + i] = inside ? -unsigned_d : unsigned_d;
                }
            }
        }
    };
    if (threads <= 1) {
        slab(0, g.nz);
    } else {
        std::vector<std::thread> pool;
        uint32_t span = (g.nz + threads - 1) / threads;
        for (unsigned t = 0; t < threads; ++t) {
            uint32_t k0 = t * span, k1 = std::min<uint32_t>((t + 1) * span, g.nz);
            if (k0 < k1) pool.emplace_back(slab, k0, k1);
        }
        for (auto& th : pool) th.join();
    }
    return "";
}

}  // namespace mesh
}  // namespace oracle
