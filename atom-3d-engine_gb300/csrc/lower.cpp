// lower.cpp — validation and lowering of an MM3E scene description into a device tape.
//
// The world plan built here is the one the reference's accelerated field uses
// (mm3e-orchestrator/src/accel.rs:134-185): maximal runs of plain-union objects become a
// bounding-sphere BVH (median split on the longest centroid axis, ties by object index),
// smooth/subtract objects become single segments, and the prune slack is the widest smooth
// radius plus 0.1. Bounds follow Object::world_bound (lib.rs:470-496). All arithmetic is
// binary32 without contraction (this file is compiled with -ffp-contract=off), so node centres
// and radii are bit-identical to the reference's and the GPU prunes exactly where it prunes.
#include "lower.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace mm3e {
namespace {

struct V {
    float x, y, z;
};
inline V vadd(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V vsub(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V vscale(V a, float s) { return V{a.x * s, a.y * s, a.z * s}; }
inline float vdot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float vlen(V a) { return std::sqrt(vdot(a, a)); }
inline V vmin(V a, V b) { return V{std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline V vmax(V a, V b) { return V{std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
inline V v3(const float* a) { return V{a[0], a[1], a[2]}; }
inline bool vzero(V a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
// Mat3::mul_vec over columns (vec.rs:125-127)
inline V mulvec(const float* rot, V v) {
    return vadd(vadd(vscale(v3(rot), v.x), vscale(v3(rot + 3), v.y)), vscale(v3(rot + 6), v.z));
}
inline bool fin(float x) { return std::isfinite(x); }
inline bool fin3(const float* a) { return fin(a[0]) && fin(a[1]) && fin(a[2]); }

// accel.rs:26-36 / csg.rs:86-97 (same arithmetic)
void enclose(V c1, float r1, V c2, float r2, V& c, float& r) {
    float d = vlen(vsub(c2, c1));
    if (d + r2 <= r1) { c = c1; r = r1; return; }
    if (d + r1 <= r2) { c = c2; r = r2; return; }
    float radius = (d + r1 + r2) * 0.5f;
    c = vadd(c1, vscale(vsub(c2, c1), (radius - r1) / std::fmax(d, 1e-12f)));
    r = radius;
}

// to_world (vec.rs:190-192)
V to_world(const float* rot, V pos, float scale, V p) { return vadd(pos, mulvec(rot, vscale(p, scale))); }

// csg.rs:120-150; false = None
bool csg_bound(const mm3e_csg_node* nodes, uint32_t i, V& c, float& r) {
    const mm3e_csg_node& n = nodes[i];
    const float* q = n.params;
    switch (n.kind) {
        case MM3E_PRIM_SPHERE: c = V{0, 0, 0}; r = q[0]; return true;
        case MM3E_PRIM_BOX:
        case MM3E_PRIM_ROUND_BOX: c = V{0, 0, 0}; r = vlen(V{q[0], q[1], q[2]}); return true;
        case MM3E_PRIM_TORUS: c = V{0, 0, 0}; r = q[0] + q[1]; return true;
        case MM3E_PRIM_CYLINDER: c = V{0, 0, 0}; r = std::sqrt(q[0] * q[0] + q[1] * q[1]); return true;
        case MM3E_PRIM_CAPSULE: {
            V a{q[0], q[1], q[2]}, b{q[3], q[4], q[5]};
            c = vscale(vadd(a, b), 0.5f);
            r = vlen(vsub(a, b)) * 0.5f + q[6];
            return true;
        }
        case MM3E_PRIM_CONE: c = V{0, q[2] * 0.5f, 0}; r = q[2] * 0.5f + std::fmax(q[0], q[1]); return true;
        case MM3E_PRIM_ELLIPSOID:
        case MM3E_PRIM_OCTAHEDRON:
        case MM3E_PRIM_PLANE: return false;
        case MM3E_PRIM_HEX_PRISM: c = V{0, 0, 0}; r = std::sqrt(4.0f * q[0] * q[0] / 3.0f + q[1] * q[1]); return true;
        case MM3E_CSG_TRANSFORM: {
            V cc;
            float rr;
            if (!csg_bound(nodes, n.a, cc, rr)) return false;
            c = to_world(n.rot, v3(n.pos), n.scale, cc);
            r = rr * n.scale;
            return true;
        }
        case MM3E_CSG_UNION:
        case MM3E_CSG_SMOOTH_UNION: {
            V ac, bc;
            float ar, br;
            if (!csg_bound(nodes, n.a, ac, ar)) return false;
            if (!csg_bound(nodes, n.b, bc, br)) return false;
            enclose(ac, ar, bc, br, c, r);
            if (n.kind == MM3E_CSG_SMOOTH_UNION) r = r + q[0] * 0.25f;
            return true;
        }
        case MM3E_CSG_INTERSECT: {
            V ac, bc;
            float ar, br;
            bool ha = csg_bound(nodes, n.a, ac, ar), hb = csg_bound(nodes, n.b, bc, br);
            if (ha && hb) {
                if (ar <= br) { c = ac; r = ar; } else { c = bc; r = br; }
                return true;
            }
            if (ha) { c = ac; r = ar; return true; }
            if (hb) { c = bc; r = br; return true; }
            return false;
        }
        case MM3E_CSG_SUBTRACT: return csg_bound(nodes, n.a, c, r);
        case MM3E_CSG_OFFSET:
            if (!csg_bound(nodes, n.a, c, r)) return false;
            r = std::fmax(r + q[0], 0.0f);
            return true;
        case MM3E_CSG_SHELL:
            if (!csg_bound(nodes, n.a, c, r)) return false;
            r = r + q[0];
            return true;
        default: return false;
    }
}

// csg.rs:154-236 (Expr::validate_at). Nested rotations are composed as a plain matrix
// product for the cumulative-position limit check.
int csg_validate(const mm3e_scene_desc& d, uint32_t i, uint32_t depth, uint32_t& count, const float* prot, V ppos,
                 float pscale, std::string& err) {
    if (i >= d.n_csg_nodes) {
        err = "CSG node index out of range";
        return MM3E_ERR_INVALID;
    }
    count += 1;
    if (depth > 64 || count > 1024) {
        err = "CSG expression exceeds depth/node budget";
        return MM3E_ERR_INVALID;
    }
    const mm3e_csg_node& n = d.csg_nodes[i];
    const float* q = n.params;
    auto positive = [](float x) { return fin(x) && x >= 1e-6f && x <= 1e6f; };
    auto scalar = [](float x) { return fin(x) && std::fabs(x) <= 1e6f; };
    auto finite3 = [&](V v) { return scalar(v.x) && scalar(v.y) && scalar(v.z); };
    auto extents = [&](V v) { return positive(v.x) && positive(v.y) && positive(v.z); };
    bool good = true;
    switch (n.kind) {
        case MM3E_PRIM_SPHERE: good = positive(q[0]); break;
        case MM3E_PRIM_BOX: good = extents(V{q[0], q[1], q[2]}); break;
        case MM3E_PRIM_ROUND_BOX:
            good = extents(V{q[0], q[1], q[2]}) && scalar(q[3]) && q[3] >= 0.0f &&
                   q[3] <= std::fmin(std::fmin(q[0], q[1]), q[2]);
            break;
        case MM3E_PRIM_TORUS: good = positive(q[0]) && positive(q[1]) && q[1] <= q[0]; break;
        case MM3E_PRIM_CYLINDER: good = positive(q[0]) && positive(q[1]); break;
        case MM3E_PRIM_CAPSULE:
            good = finite3(V{q[0], q[1], q[2]}) && finite3(V{q[3], q[4], q[5]}) && positive(q[6]) &&
                   vlen(vsub(V{q[0], q[1], q[2]}, V{q[3], q[4], q[5]})) >= 1e-6f;
            break;
        case MM3E_PRIM_CONE:
            good = positive(q[2]) && scalar(q[0]) && scalar(q[1]) && q[0] >= 0.0f && q[1] >= 0.0f &&
                   std::fmax(q[0], q[1]) > 0.0f && std::fabs(q[0] - q[1]) < q[2];
            break;
        case MM3E_PRIM_ELLIPSOID: good = extents(V{q[0], q[1], q[2]}); break;
        case MM3E_PRIM_OCTAHEDRON: good = positive(q[0]); break;
        case MM3E_PRIM_HEX_PRISM: good = positive(q[0]) && positive(q[1]); break;
        case MM3E_PRIM_PLANE:
            good = finite3(V{q[0], q[1], q[2]}) && scalar(q[3]) && std::fabs(vlen(V{q[0], q[1], q[2]}) - 1.0f) <= 1e-5f;
            break;
        case MM3E_CSG_TRANSFORM: {
            V c0 = v3(n.rot), c1 = v3(n.rot + 3), c2 = v3(n.rot + 6);
            auto unit = [&](V c) { return finite3(c) && std::fabs(vlen(c) - 1.0f) <= 1e-5f; };
            V cr{c0.y * c1.z - c0.z * c1.y, c0.z * c1.x - c0.x * c1.z, c0.x * c1.y - c0.y * c1.x};
            bool rotation = unit(c0) && unit(c1) && unit(c2) && std::fabs(vdot(c0, c1)) <= 1e-5f &&
                            std::fabs(vdot(c0, c2)) <= 1e-5f && std::fabs(vdot(c1, c2)) <= 1e-5f &&
                            std::fabs(vdot(cr, c2) - 1.0f) <= 1e-5f;
            if (!finite3(v3(n.pos)) || !positive(n.scale) || !rotation) {
                err = "CSG transform requires finite position, positive scale and a proper orthonormal rotation";
                return MM3E_ERR_INVALID;
            }
            V cpos = to_world(prot, ppos, pscale, v3(n.pos));
            float cscale = pscale * n.scale;
            float crot[9];
            for (int c = 0; c < 3; ++c) {
                V col = mulvec(prot, v3(n.rot + 3 * c));
                crot[3 * c] = col.x;
                crot[3 * c + 1] = col.y;
                crot[3 * c + 2] = col.z;
            }
            if (!positive(cscale) || !finite3(cpos)) {
                err = "CSG cumulative transform exceeds finite coordinate/scale limits";
                return MM3E_ERR_INVALID;
            }
            int rc = csg_validate(d, n.a, depth + 1, count, crot, cpos, cscale, err);
            if (rc) return rc;
            break;
        }
        case MM3E_CSG_UNION:
        case MM3E_CSG_INTERSECT:
        case MM3E_CSG_SUBTRACT:
        case MM3E_CSG_SMOOTH_UNION: {
            if (n.kind == MM3E_CSG_SMOOTH_UNION && (!scalar(q[0]) || q[0] < 0.0f)) {
                err = "CSG smooth radius must be finite and nonnegative";
                return MM3E_ERR_INVALID;
            }
            int rc = csg_validate(d, n.a, depth + 1, count, prot, ppos, pscale, err);
            if (rc) return rc;
            rc = csg_validate(d, n.b, depth + 1, count, prot, ppos, pscale, err);
            if (rc) return rc;
            break;
        }
        case MM3E_CSG_OFFSET: {
            int rc = csg_validate(d, n.a, depth + 1, count, prot, ppos, pscale, err);
            if (rc) return rc;
            good = scalar(q[0]);
            break;
        }
        case MM3E_CSG_SHELL: {
            int rc = csg_validate(d, n.a, depth + 1, count, prot, ppos, pscale, err);
            if (rc) return rc;
            good = positive(q[0]);
            break;
        }
        default:
            err = "unknown CSG node kind";
            return MM3E_ERR_INVALID;
    }
    if (!good) {
        err = "invalid CSG primitive or modifier parameters";
        return MM3E_ERR_INVALID;
    }
    V bc;
    float br;
    if (csg_bound(d.csg_nodes, i, bc, br)) {
        if (!finite3(bc) || !fin(br) || !(br >= 0.0f && br <= 1e12f)) {
            err = "CSG expression has an invalid or excessive evaluated bound";
            return MM3E_ERR_INVALID;
        }
    }
    return MM3E_OK;
}

// Emits the post-order program of CSG node i; tracks value/point stack depth.
void csg_emit(const mm3e_scene_desc& d, uint32_t i, std::vector<DevCsgOp>& ops, int& vdepth, int& pdepth, int& vmax,
              int& pmax) {
    const mm3e_csg_node& n = d.csg_nodes[i];
    DevCsgOp op{};
    for (int j = 0; j < 7; ++j) op.p[j] = n.params[j];
    switch (n.kind) {
        case MM3E_CSG_TRANSFORM: {
            DevCsgOp x{};
            x.op = CSG_OP_XFORM;
            for (int j = 0; j < 9; ++j) x.rot[j] = n.rot[j];
            for (int j = 0; j < 3; ++j) x.pos[j] = n.pos[j];
            x.scale = n.scale;
            x.inv = std::fabs(n.scale) > 1e-12f ? 1.0f / n.scale : 0.0f;
            ops.push_back(x);
            pdepth += 1;
            pmax = std::max(pmax, pdepth);
            csg_emit(d, n.a, ops, vdepth, pdepth, vmax, pmax);
            DevCsgOp u = x;
            u.op = CSG_OP_UNXFORM;
            ops.push_back(u);
            pdepth -= 1;
            return;
        }
        case MM3E_CSG_UNION:
        case MM3E_CSG_INTERSECT:
        case MM3E_CSG_SUBTRACT:
        case MM3E_CSG_SMOOTH_UNION:
            csg_emit(d, n.a, ops, vdepth, pdepth, vmax, pmax);
            csg_emit(d, n.b, ops, vdepth, pdepth, vmax, pmax);
            op.op = n.kind == MM3E_CSG_UNION       ? CSG_OP_UNION
                    : n.kind == MM3E_CSG_INTERSECT ? CSG_OP_INTERSECT
                    : n.kind == MM3E_CSG_SUBTRACT  ? CSG_OP_SUBTRACT
                                                   : CSG_OP_SMOOTH;
            ops.push_back(op);
            vdepth -= 1;
            return;
        case MM3E_CSG_OFFSET:
        case MM3E_CSG_SHELL:
            csg_emit(d, n.a, ops, vdepth, pdepth, vmax, pmax);
            op.op = n.kind == MM3E_CSG_OFFSET ? CSG_OP_OFFSET : CSG_OP_SHELL;
            ops.push_back(op);
            return;
        default:
            op.op = CSG_OP_PRIM;
            op.kind = n.kind;
            ops.push_back(op);
            vdepth += 1;
            vmax = std::max(vmax, vdepth);
            return;
    }
}

// Volume bounds (volume.rs:97-103)
void volume_bounds(const mm3e_volume& v, V& lo, V& hi) {
    float sx = (float)(v.nx - 1) * v.cell[0];
    float sy = (float)(v.ny - 1) * v.cell[1];
    float sz = (float)(v.nz - 1) * v.cell[2];
    lo = v3(v.min);
    hi = vadd(lo, V{sx, sy, sz});
}

// Prim::local_bound (lib.rs:264-292); false = None
bool local_bound(const mm3e_scene_desc& d, const mm3e_object& o, V& c, float& r) {
    const float* q = o.params;
    switch (o.prim) {
        case MM3E_PRIM_SPHERE: c = V{0, 0, 0}; r = q[0]; return true;
        case MM3E_PRIM_BOX:
        case MM3E_PRIM_ROUND_BOX: c = V{0, 0, 0}; r = vlen(V{q[0], q[1], q[2]}); return true;
        case MM3E_PRIM_TORUS: c = V{0, 0, 0}; r = q[0] + q[1]; return true;
        case MM3E_PRIM_CYLINDER: c = V{0, 0, 0}; r = std::sqrt(q[0] * q[0] + q[1] * q[1]); return true;
        case MM3E_PRIM_CAPSULE: {
            V a{q[0], q[1], q[2]}, b{q[3], q[4], q[5]};
            c = vscale(vadd(a, b), 0.5f);
            r = vlen(vscale(vsub(a, b), 0.5f)) + q[6];
            return true;
        }
        case MM3E_PRIM_CONE:
            c = V{0, q[2] * 0.5f, 0};
            r = std::fmax(std::fmax(q[2] * 0.5f + std::fmax(q[0], q[1]), q[0]), q[1]);
            return true;
        case MM3E_PRIM_ELLIPSOID: c = V{0, 0, 0}; r = std::fmax(std::fmax(q[0], q[1]), q[2]); return true;
        case MM3E_PRIM_OCTAHEDRON: c = V{0, 0, 0}; r = q[0]; return true;
        case MM3E_PRIM_HEX_PRISM: c = V{0, 0, 0}; r = std::sqrt(q[0] * q[0] + q[1] * q[1]); return true;
        case MM3E_PRIM_PLANE: return false;
        case MM3E_PRIM_CSG: return csg_bound(d.csg_nodes, d.csg_roots[o.id], c, r);
        case MM3E_PRIM_VOLUME: {
            if (d.n_volumes == 0) return false;
            V lo, hi;
            volume_bounds(d.volumes[o.id % d.n_volumes], lo, hi);
            c = vscale(vadd(lo, hi), 0.5f);
            r = vlen(vscale(vsub(hi, lo), 0.5f));
            return true;
        }
        default: return false;
    }
}

// Object::world_bound (lib.rs:470-496)
bool world_bound(const mm3e_scene_desc& d, const mm3e_object& o, V& wc, float& wr) {
    V center;
    float radius;
    if (!local_bound(d, o, center, radius)) return false;
    if (!vzero(v3(o.repeat)) || o.bend != 0.0f) return false;
    if (o.mirror & 7u) {
        radius = radius + vlen(center);
        center = V{0, 0, 0};
    }
    if (o.twist != 0.0f) {
        radius = radius + std::sqrt(center.x * center.x + center.z * center.z);
        center.x = 0.0f;
        center.z = 0.0f;
    }
    radius = radius + vlen(v3(o.elongate));
    wc = vadd(v3(o.pos), mulvec(o.rot, vscale(center, o.scale)));
    wr = radius * o.scale + std::fmax(o.round, 0.0f) + std::fabs(o.onion);
    return true;
}

struct Item {
    uint32_t index;
    V c;
    float r;
};

// accel.rs:39-77
uint32_t bvh_build(Item* items, size_t n, std::vector<DevNode>& nodes, uint32_t depth, uint32_t& max_depth) {
    max_depth = std::max(max_depth, depth);
    if (n == 1) {
        nodes.push_back(DevNode{items[0].c.x, items[0].c.y, items[0].c.z, items[0].r, 0, 0, (int32_t)items[0].index, 0});
        return (uint32_t)(nodes.size() - 1);
    }
    float inf = INFINITY;
    V lo{inf, inf, inf}, hi{-inf, -inf, -inf};
    for (size_t i = 0; i < n; ++i) {
        lo = vmin(lo, items[i].c);
        hi = vmax(hi, items[i].c);
    }
    V ext = vsub(hi, lo);
    int axis = (ext.x >= ext.y && ext.x >= ext.z) ? 0 : (ext.y >= ext.z ? 1 : 2);
    auto coord = [axis](const V& c) { return axis == 0 ? c.x : (axis == 1 ? c.y : c.z); };
    std::sort(items, items + n, [&](const Item& a, const Item& b) {
        float ca = coord(a.c), cb = coord(b.c);
        if (ca < cb) return true;
        if (ca > cb) return false;
        return a.index < b.index;
    });
    size_t mid = n / 2;
    uint32_t left = bvh_build(items, mid, nodes, depth + 1, max_depth);
    uint32_t right = bvh_build(items + mid, n - mid, nodes, depth + 1, max_depth);
    V c;
    float r;
    enclose(V{nodes[left].cx, nodes[left].cy, nodes[left].cz}, nodes[left].r,
            V{nodes[right].cx, nodes[right].cy, nodes[right].cz}, nodes[right].r, c, r);
    nodes.push_back(DevNode{c.x, c.y, c.z, r, (int32_t)left, (int32_t)right, -1, 0});
    return (uint32_t)(nodes.size() - 1);
}

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

}  // namespace

// Gaussian kernel of post.rs:331-345 in binary32 (host libm expf, as the reference).
std::vector<float> gaussian_kernel(uint32_t radius) {
    int32_t r = (int32_t)(radius > 1 ? radius : 1);
    float sigma = std::fmax((float)r / 2.0f, 1e-3f);
    std::vector<float> k;
    float sum = 0.0f;
    for (int32_t i = -r; i <= r; ++i) {
        float v = expf((float)(-(i * i)) / (2.0f * sigma * sigma));
        k.push_back(v);
        sum = sum + v;
    }
    for (auto& v : k) v = v / sum;
    return k;
}

bool gi_setup(const mm3e_scene_desc& d, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t samples, GiSetup& out) {
    float inf = INFINITY;
    V lo{inf, inf, inf}, hi{-inf, -inf, -inf};
    bool any = false;
    for (uint32_t i = 0; i < d.n_objects; ++i) {
        V c;
        float r;
        if (!world_bound(d, d.objects[i], c, r)) continue;
        any = true;
        lo = vmin(lo, vsub(c, V{r, r, r}));
        hi = vmax(hi, vadd(c, V{r, r, r}));
    }
    if (!any) return false;
    lo = vsub(lo, V{1.5f, 1.5f, 1.5f});
    hi = vadd(hi, V{1.5f, 1.5f, 1.5f});
    out.nx = nx > 1 ? nx : 1;
    out.ny = ny > 1 ? ny : 1;
    out.nz = nz > 1 ? nz : 1;
    V size = vsub(hi, lo);
    auto den = [](uint32_t n) { return (float)((n > 2 ? n : 2) - 1); };
    V cell{size.x / den(out.nx), size.y / den(out.ny), size.z / den(out.nz)};
    out.lo[0] = lo.x; out.lo[1] = lo.y; out.lo[2] = lo.z;
    out.size[0] = size.x; out.size[1] = size.y; out.size[2] = size.z;
    out.cell[0] = cell.x; out.cell[1] = cell.y; out.cell[2] = cell.z;
    out.dirs_per_face = samples > 1 ? 5u : 1u;
    out.dirs.clear();
    const V axes[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    auto normalize = [](V a) {
        float len = vlen(a);
        return len > 1e-12f ? vscale(a, 1.0f / len) : V{0, 0, 0};
    };
    auto cross = [](V a, V o) { return V{a.y * o.z - a.z * o.y, a.z * o.x - a.x * o.z, a.x * o.y - a.y * o.x}; };
    for (const V& axis : axes) {
        V up = std::fabs(axis.y) > 0.9f ? V{1, 0, 0} : V{0, 1, 0};
        V t1 = normalize(cross(axis, up));
        V t2 = normalize(cross(axis, t1));
        out.dirs.insert(out.dirs.end(), {axis.x, axis.y, axis.z, 1.0f});
        if (samples > 1) {
            V ts[4] = {t1, t2, vscale(t1, -1.0f), vscale(t2, -1.0f)};
            for (const V& t : ts) {
                V dd = normalize(vadd(vscale(axis, 0.72f), vscale(t, 0.72f)));
                out.dirs.insert(out.dirs.end(), {dd.x, dd.y, dd.z, std::fmax(vdot(dd, axis), 0.0f)});
            }
        }
    }
    return true;
}

int validate_scene(const mm3e_scene_desc& d, std::string& err) {
    if (d.width > 16384 || d.height > 16384) {
        err = "render dimensions must be at most 16384";
        return MM3E_ERR_INVALID;
    }
    if (d.n_materials == 0 || d.materials == nullptr) {
        err = "scene needs at least one material";
        return MM3E_ERR_INVALID;
    }
    if ((d.n_objects && !d.objects) || (d.n_lights && !d.lights)) {
        err = "null object or light array";
        return MM3E_ERR_INVALID;
    }
    if (d.mode > MM3E_MODE_ALBEDO) {
        err = "unknown render mode";
        return MM3E_ERR_INVALID;
    }
    if (d.aa > (uint32_t)MAX_AA) {
        err = "aa must be at most 16";
        return MM3E_ERR_UNSUPPORTED;
    }
    if (d.bounces > (uint32_t)MAX_BOUNCES) {
        err = "bounces must be at most 7";
        return MM3E_ERR_UNSUPPORTED;
    }
    if (d.post.bloom && d.post.bloom_intensity > 0.0f && d.post.bloom_radius > MAX_BLOOM_RADIUS) {
        // every output pixel sums 2r+1 taps per blur pass: a larger kernel would hold the GPU for minutes
        err = "bloom radius must be at most 4096";
        return MM3E_ERR_UNSUPPORTED;
    }
    if (d.n_csgs && (!d.csg_roots || !d.csg_nodes)) {
        err = "null CSG arrays";
        return MM3E_ERR_INVALID;
    }
    for (uint32_t e = 0; e < d.n_csgs; ++e) {
        uint32_t count = 0;
        const float ident[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        int rc = csg_validate(d, d.csg_roots[e], 1, count, ident, V{0, 0, 0}, 1.0f, err);
        if (rc) return rc;
        std::vector<DevCsgOp> ops;
        int vd = 0, pd = 0, vm = 0, pm = 0;
        csg_emit(d, d.csg_roots[e], ops, vd, pd, vm, pm);
        if (vm > MAX_CSG_STACK || pm > MAX_CSG_STACK) {
            err = "CSG expression needs a deeper evaluation stack than this path supports (16)";
            return MM3E_ERR_UNSUPPORTED;
        }
    }
    for (uint32_t i = 0; i < d.n_volumes; ++i) {
        const mm3e_volume& v = d.volumes[i];
        if (v.nx < 2 || v.ny < 2 || v.nz < 2) {
            err = "SdfVolume dims must all be >= 2";
            return MM3E_ERR_INVALID;
        }
        if (!fin3(v.min)) {
            err = "SdfVolume min must be finite";
            return MM3E_ERR_INVALID;
        }
        if (!fin3(v.cell) || !(v.cell[0] > 0 && v.cell[1] > 0 && v.cell[2] > 0)) {
            err = "SdfVolume cell sizes must be positive and finite";
            return MM3E_ERR_INVALID;
        }
        if (!v.data) {
            err = "SdfVolume data is null";
            return MM3E_ERR_INVALID;
        }
        uint64_t n = (uint64_t)v.nx * v.ny * v.nz;
        for (uint64_t j = 0; j < n; ++j)
            if (!fin(v.data[j])) {
                err = "SdfVolume sample " + std::to_string(j) + " is non-finite";
                return MM3E_ERR_INVALID;
            }
    }
    if (d.gi) {
        if (d.gi->nx == 0 || d.gi->ny == 0 || d.gi->nz == 0 || !d.gi->cubes) {
            err = "GI volume needs at least one probe per axis and cube data";
            return MM3E_ERR_INVALID;
        }
    }
    for (uint32_t i = 0; i < d.n_objects; ++i) {
        const mm3e_object& o = d.objects[i];
        if (o.prim == MM3E_PRIM_SURFACE) {
            err = "native triangle surfaces are not supported by the GPU backend; use the CPU renderer";
            return MM3E_ERR_UNSUPPORTED;
        }
        if (o.prim > MM3E_PRIM_VOLUME) {
            err = "object " + std::to_string(i) + ": unknown primitive";
            return MM3E_ERR_INVALID;
        }
        if (o.prim == MM3E_PRIM_CSG && o.id >= d.n_csgs) {
            err = "unregistered CSG expression";
            return MM3E_ERR_INVALID;
        }
        if (o.combine > MM3E_COMBINE_SUBTRACT) {
            err = "object " + std::to_string(i) + ": unknown combine mode";
            return MM3E_ERR_INVALID;
        }
        bool ok = fin3(o.pos) && fin(o.scale) && fin(o.smooth_k);
        for (int j = 0; j < 9; ++j) ok = ok && fin(o.rot[j]);
        for (int j = 0; j < 7; ++j) ok = ok && fin(o.params[j]);
        ok = ok && fin3(o.repeat) && fin3(o.elongate) && fin(o.twist) && fin(o.bend) && fin(o.round) && fin(o.onion);
        if (!ok) {
            err = "object " + std::to_string(i) + ": transform, parameters and modifiers must be finite";
            return MM3E_ERR_INVALID;
        }
    }
    return MM3E_OK;
}

int validate_dynamic(const mm3e_scene_desc& d, const mm3e_dyn_sphere* dyn, size_t n, std::string& err) {
    for (size_t i = 0; i < n; ++i) {
        const mm3e_dyn_sphere& s = dyn[i];
        if (!fin3(s.pos)) {
            err = "dynamic sphere " + std::to_string(i) + ": position must be finite";
            return MM3E_ERR_INVALID;
        }
        if (!fin(s.radius) || s.radius <= 0.0f) {
            err = "dynamic sphere " + std::to_string(i) + ": radius must be finite and positive";
            return MM3E_ERR_INVALID;
        }
        float v[4] = {s.albedo[0], s.albedo[1], s.albedo[2], s.metallic};
        for (float x : v)
            if (!fin(x) || x < 0.0f || x > 1.0f) {
                err = "dynamic sphere " + std::to_string(i) + ": linear albedo and metallic must be finite and in [0,1]";
                return MM3E_ERR_INVALID;
            }
    }
    if ((uint64_t)d.n_materials + n > 0xFFFFFFFFull) {
        err = "dynamic spheres exceed material ID capacity";
        return MM3E_ERR_INVALID;
    }
    return MM3E_OK;
}

int lower_scene(const mm3e_scene_desc& d0, const mm3e_dyn_sphere* dyn, size_t n_dyn, LoweredScene& out,
                std::string& err) {
    int rc = validate_scene(d0, err);
    if (rc) return rc;
    rc = validate_dynamic(d0, dyn, n_dyn, err);
    if (rc) return rc;

    // Snapshot with dynamic spheres appended (mm3e-cpu-parallel/src/lib.rs:58-64).
    std::vector<mm3e_object> objects(d0.objects, d0.objects + d0.n_objects);
    std::vector<mm3e_material> materials(d0.materials, d0.materials + d0.n_materials);
    for (size_t i = 0; i < n_dyn; ++i) {
        mm3e_material m{};
        m.albedo[0] = dyn[i].albedo[0];
        m.albedo[1] = dyn[i].albedo[1];
        m.albedo[2] = dyn[i].albedo[2];
        m.metallic = dyn[i].metallic;
        m.specular = 0.5f;
        m.roughness = 0.35f;
        materials.push_back(m);
        mm3e_object o{};
        o.prim = MM3E_PRIM_SPHERE;
        o.params[0] = dyn[i].radius;
        o.rot[0] = o.rot[4] = o.rot[8] = 1.0f;
        o.pos[0] = dyn[i].pos[0];
        o.pos[1] = dyn[i].pos[1];
        o.pos[2] = dyn[i].pos[2];
        o.scale = 1.0f;
        o.mat = (uint32_t)(materials.size() - 1);
        o.combine = MM3E_COMBINE_UNION;
        objects.push_back(o);
    }
    mm3e_scene_desc d = d0;
    d.objects = objects.data();
    d.n_objects = (uint32_t)objects.size();
    d.materials = materials.data();
    d.n_materials = (uint32_t)materials.size();

    const uint32_t n = d.n_objects;
    // World bounds and slack (accel.rs:140-148).
    std::vector<DevObject> objs(n);
    std::vector<bool> has_bound(n);
    std::vector<V> bc(n);
    std::vector<float> br(n);
    float mk = 0.0f;
    bool dual_safe = true;
    for (uint32_t i = 0; i < n; ++i) {
        const mm3e_object& o = d.objects[i];
        has_bound[i] = world_bound(d, o, bc[i], br[i]);
        mk = std::fmax(mk, o.combine == MM3E_COMBINE_SMOOTH ? o.smooth_k : 0.0f);
        if (o.twist != 0.0f || o.bend != 0.0f || o.prim == MM3E_PRIM_VOLUME || o.prim == MM3E_PRIM_CSG)
            dual_safe = false;
    }
    float slack = mk + 0.1f;

    // CSG programs
    std::vector<DevCsgOp> csg_ops;
    std::vector<uint32_t> csg_offset(d.n_csgs);
    int csg_stack = 0;
    for (uint32_t e = 0; e < d.n_csgs; ++e) {
        csg_offset[e] = (uint32_t)csg_ops.size();
        int vd = 0, pd = 0, vm = 0, pm = 0;
        csg_emit(d, d.csg_roots[e], csg_ops, vd, pd, vm, pm);
        DevCsgOp end{};
        end.op = CSG_OP_END;
        csg_ops.push_back(end);
        csg_stack = std::max(csg_stack, std::max(vm, pm));
    }

    for (uint32_t i = 0; i < n; ++i) {
        const mm3e_object& o = d.objects[i];
        DevObject& g = objs[i];
        std::memset(&g, 0, sizeof(g));
        std::memcpy(g.rot, o.rot, sizeof(g.rot));
        std::memcpy(g.pos, o.pos, sizeof(g.pos));
        g.scale = o.scale;
        g.inv = std::fabs(o.scale) > 1e-12f ? 1.0f / o.scale : 0.0f;
        std::memcpy(g.params, o.params, sizeof(g.params));
        g.prim = o.prim;
        g.mat = o.mat;
        g.k = o.smooth_k;
        uint32_t f = o.mirror & 7u;
        if (!vzero(v3(o.elongate))) f |= OF_ELONGATE;
        if (!vzero(v3(o.repeat))) f |= OF_REPEAT;
        if (o.twist != 0.0f) f |= OF_TWIST;
        if (o.bend != 0.0f) f |= OF_BEND;
        if (o.round != 0.0f) f |= OF_ROUND;
        if (o.onion != 0.0f) f |= OF_ONION;
        if (has_bound[i]) f |= OF_BOUND;
        // Fields that can lie below their bounding sphere's distance: the ellipsoid and octahedron
        // bound fields, and the hexagonal prism, whose Prim::local_bound radius (lib.rs:264-292)
        // takes the hexagon's apothem where its corners reach 2/sqrt(3) times as far.
        if (o.prim == MM3E_PRIM_ELLIPSOID || o.prim == MM3E_PRIM_OCTAHEDRON || o.prim == MM3E_PRIM_HEX_PRISM)
            f |= OF_NONCONS;
        {
            static const float ident[9] = {1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f};
            if (std::memcmp(o.rot, ident, sizeof(ident)) == 0) f |= OF_ROT_IDENTITY;  // bitwise: no -0 entries
        }
        f |= (o.combine & 3u) << 16;  // combine mode, read by the dual-number normal
        g.flags = f;
        g.aux = o.prim == MM3E_PRIM_CSG ? csg_offset[o.id] : (d.n_volumes ? o.id % d.n_volumes : 0);
        std::memcpy(g.elongate, o.elongate, sizeof(g.elongate));
        std::memcpy(g.repeat, o.repeat, sizeof(g.repeat));
        g.twist = o.twist;
        g.bend = o.bend;
        g.round = o.round;
        g.onion = o.onion;
        g.bc[0] = bc[i].x;
        g.bc[1] = bc[i].y;
        g.bc[2] = bc[i].z;
        g.br = br[i];
        if (o.prim == MM3E_PRIM_VOLUME && d.n_volumes == 0) g.prim = 0xFFu;  // distance = +inf
    }

    // World plan segments (accel.rs:150-184)
    std::vector<DevSegment> segs;
    std::vector<DevNode> nodes;
    std::vector<uint32_t> unbounded;
    uint32_t max_depth = 0;
    std::vector<uint32_t> run;
    auto close_run = [&]() {
        if (run.empty()) return;
        std::vector<Item> items;
        DevSegment s{SEG_RUN, 0, 0, NIL, 0, 0, 0, 0};
        if (run.size() <= LINEAR_MAX) {
            s.kind = SEG_LINEAR;
            s.a = (uint32_t)unbounded.size();
            s.b = (uint32_t)run.size();
            for (uint32_t i : run) unbounded.push_back(i);
        }
        s.ua = (uint32_t)unbounded.size();
        for (uint32_t i : run) {
            if (has_bound[i]) items.push_back(Item{i, bc[i], br[i]});
            else unbounded.push_back(i);
        }
        s.ub = (uint32_t)unbounded.size() - s.ua;
        if (!items.empty()) {
            std::vector<DevNode> local;
            uint32_t root = bvh_build(items.data(), items.size(), local, 1, max_depth);
            uint32_t base = (uint32_t)nodes.size();
            for (auto& nd : local) {
                if (nd.leaf < 0) {
                    nd.left += (int32_t)base;
                    nd.right += (int32_t)base;
                }
                nodes.push_back(nd);
            }
            s.c = base + root;
        }
        segs.push_back(s);
        run.clear();
    };
    for (uint32_t i = 0; i < n; ++i) {
        if (d.objects[i].combine == MM3E_COMBINE_UNION) {
            run.push_back(i);
        } else {
            close_run();
            segs.push_back(DevSegment{SEG_ONE, i, d.objects[i].combine, 0, 0, 0, 0, 0});
        }
    }
    close_run();
    // Near-first traversal pushes two entries per internal node visited: depth + 1 slots.
    if (max_depth + 1 > (uint32_t)MAX_BVH_STACK || nodes.size() > MAX_NODES) {
        err = "a plain-union run is too large for this path's traversal stack (about 2000 objects)";
        return MM3E_ERR_UNSUPPORTED;
    }

    std::vector<DevMaterial> mats(d.n_materials);
    for (uint32_t i = 0; i < d.n_materials; ++i) {
        const mm3e_material& m = d.materials[i];
        DevMaterial& g = mats[i];
        std::memset(&g, 0, sizeof(g));
        std::memcpy(g.albedo, m.albedo, sizeof(g.albedo));
        g.metallic = m.metallic;
        g.specular = m.specular;
        g.roughness = m.roughness;
        g.reflectivity = m.reflectivity;
        std::memcpy(g.emissive, m.emissive, sizeof(g.emissive));
        g.checker = m.checker ? 1u : 0u;
    }
    std::vector<DevLight> lights(d.n_lights);
    for (uint32_t i = 0; i < d.n_lights; ++i) {
        const mm3e_light& l = d.lights[i];
        std::memset(&lights[i], 0, sizeof(DevLight));
        std::memcpy(lights[i].vec, l.vec, sizeof(l.vec));
        std::memcpy(lights[i].color, l.color, sizeof(l.color));
        lights[i].directional = l.directional ? 1u : 0u;
        lights[i].radius = l.radius;
    }
    std::vector<DevVolume> vols(d.n_volumes);
    for (uint32_t i = 0; i < d.n_volumes; ++i) {
        const mm3e_volume& v = d.volumes[i];
        DevVolume& g = vols[i];
        std::memset(&g, 0, sizeof(g));
        g.nx = v.nx;
        g.ny = v.ny;
        g.nz = v.nz;
        g.valid = 1;
        std::memcpy(g.min, v.min, sizeof(g.min));
        std::memcpy(g.cell, v.cell, sizeof(g.cell));
        V lo, hi;
        volume_bounds(v, lo, hi);
        g.hi[0] = hi.x;
        g.hi[1] = hi.y;
        g.hi[2] = hi.z;
    }

    // Assemble the blob.
    TapeHeader h;
    std::memset(&h, 0, sizeof(h));
    size_t off = align16(sizeof(TapeHeader));
    auto place = [&](size_t bytes) {
        size_t o = off;
        off = align16(off + bytes);
        return (uint32_t)o;
    };
    h.off_objects = place(objs.size() * sizeof(DevObject));
    h.off_materials = place(mats.size() * sizeof(DevMaterial));
    h.off_lights = place(lights.size() * sizeof(DevLight));
    h.off_segments = place(segs.size() * sizeof(DevSegment));
    h.off_nodes = place(nodes.size() * sizeof(DevNode));
    h.off_unbounded = place(unbounded.size() * sizeof(uint32_t));
    h.off_csg = place(csg_ops.size() * sizeof(DevCsgOp));
    h.off_volumes = place(vols.size() * sizeof(DevVolume));
    size_t total = off;
    h.magic = TAPE_MAGIC;
    h.bytes = (uint32_t)total;
    h.n_objects = n;
    h.n_materials = d.n_materials;
    h.n_lights = d.n_lights;
    h.n_segments = (uint32_t)segs.size();
    h.n_nodes = (uint32_t)nodes.size();
    h.n_unbounded = (uint32_t)unbounded.size();
    h.n_csg_ops = (uint32_t)csg_ops.size();
    h.n_volumes = d.n_volumes;
    h.width = d.width;
    h.height = d.height;
    h.aa = d.aa > 1 ? d.aa : 1;
    h.bounces = d.bounces;
    h.mode = d.mode;
    uint32_t flags = 0;
    if (d.shadows) flags |= SF_SHADOWS;
    if (d.ao) flags |= SF_AO;
    if (dual_safe) flags |= SF_DUAL_SAFE;
    if (d.gi) flags |= SF_GI;
    if (d.post.bloom && d.post.bloom_intensity > 0.0f) flags |= SF_BLOOM;
    if (d.marcher.secant) flags |= SF_SECANT;
    h.flags = flags;
    h.max_steps = d.marcher.max_steps;
    h.shadow_steps = d.marcher.shadow_steps;
    h.ao_samples = d.marcher.ao_samples;
    h.max_dist = d.marcher.max_dist;
    h.eps = d.marcher.eps;
    h.step_scale = d.marcher.step_scale;
    h.lod_footprint = d.marcher.lod_footprint;
    h.subitize = d.marcher.subitize;
    h.normal_h = d.marcher.normal_h;
    h.slack = slack;
    h.fog_density = d.fog_density;
    std::memcpy(h.sun_dir, d.sun_dir, 12);
    std::memcpy(h.ambient, d.ambient, 12);
    std::memcpy(h.sky_ambient, d.sky_ambient, 12);
    std::memcpy(h.fog, d.fog, 12);
    h.exposure = d.post.exposure;
    h.bloom_threshold = d.post.bloom_threshold;
    h.bloom_intensity = d.post.bloom_intensity;
    h.bloom_radius = d.post.bloom_radius;
    out.payloads.clear();
    out.gi_float4.clear();
    if (d.gi) {
        std::memcpy(h.gi_min, d.gi->min, 12);
        std::memcpy(h.gi_size, d.gi->size, 12);
        h.gi_nx = d.gi->nx;
        h.gi_ny = d.gi->ny;
        h.gi_nz = d.gi->nz;
        size_t probes = (size_t)d.gi->nx * d.gi->ny * d.gi->nz;
        out.gi_float4.assign(probes * 24, 0.0f);
        for (size_t p = 0; p < probes; ++p)
            for (int f = 0; f < 6; ++f)
                for (int c = 0; c < 3; ++c) out.gi_float4[p * 24 + f * 4 + c] = d.gi->cubes[p * 18 + f * 3 + c];
        out.payloads.push_back({out.gi_float4.data(), out.gi_float4.size() * sizeof(float), offsetof(TapeHeader, gi_cubes)});
    }
    for (uint32_t i = 0; i < d.n_volumes; ++i) {
        const mm3e_volume& v = d.volumes[i];
        size_t bytes = (size_t)v.nx * v.ny * v.nz * sizeof(float);
        out.payloads.push_back({v.data, bytes, h.off_volumes + i * sizeof(DevVolume) + offsetof(DevVolume, data)});
    }

    out.blob.assign(total, 0);
    std::memcpy(out.blob.data(), &h, sizeof(h));
    auto put = [&](uint32_t o, const void* src, size_t bytes) {
        if (bytes) std::memcpy(out.blob.data() + o, src, bytes);
    };
    put(h.off_objects, objs.data(), objs.size() * sizeof(DevObject));
    put(h.off_materials, mats.data(), mats.size() * sizeof(DevMaterial));
    put(h.off_lights, lights.data(), lights.size() * sizeof(DevLight));
    put(h.off_segments, segs.data(), segs.size() * sizeof(DevSegment));
    put(h.off_nodes, nodes.data(), nodes.size() * sizeof(DevNode));
    put(h.off_unbounded, unbounded.data(), unbounded.size() * sizeof(uint32_t));
    put(h.off_csg, csg_ops.data(), csg_ops.size() * sizeof(DevCsgOp));
    put(h.off_volumes, vols.data(), vols.size() * sizeof(DevVolume));

    out.width = d.width;
    out.height = d.height;
    out.mode = d.mode;
    out.aa = h.aa;
    out.bounces = d.bounces;
    out.dual_safe = dual_safe;
    out.has_gi = d.gi != nullptr;
    out.bvh_depth = max_depth;
    out.csg_stack = (uint32_t)csg_stack;
    return MM3E_OK;
}

}  // namespace mm3e
