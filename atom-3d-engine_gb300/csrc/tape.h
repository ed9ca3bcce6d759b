// tape.h — device-resident scene tape: the flat lowering of an MM3E scene.
//
// One contiguous, 16-byte-aligned blob per scene holds everything a field evaluation touches:
// the world-plan segments (accel.rs WorldPlan), the bounding-sphere BVH nodes of every
// plain-union run, the object records (transform + domain modifiers + primitive parameters +
// world bound), the materials, the lights, and the post-order programs of the object-local
// CSG expressions. Render kernels copy the whole blob into shared memory once per CTA
// (cp.async.bulk) and interpret it from there. Large payloads (SDF volume samples, GI probe
// cubes) stay in global memory and are referenced by device address.
#pragma once
#ifndef __CUDACC_RTC__
#include <stdint.h>
#include <vector_types.h>
#endif

namespace mm3e {

constexpr uint32_t TAPE_MAGIC = 0x4D334554u;  // "TE3M"
constexpr uint32_t NIL = 0xFFFFFFFFu;
constexpr int MAX_BVH_STACK = 12;   // register traversal stack (16-bit node ids); host rejects deeper trees
constexpr uint32_t MAX_NODES = 65535;
constexpr int MAX_CSG_STACK = 16;   // value / point stack of a CSG program
constexpr int MAX_BOUNCES = 7;      // reflection recursion depth the kernels carry
constexpr int MAX_AA = 16;
constexpr uint32_t MAX_BLOOM_RADIUS = 4096;  // bloom kernels of at most 2 * 4096 + 1 taps

// Object flags
enum : uint32_t {
    OF_MIRROR_X = 1u << 0,
    OF_MIRROR_Y = 1u << 1,
    OF_MIRROR_Z = 1u << 2,
    OF_ELONGATE = 1u << 3,
    OF_REPEAT = 1u << 4,
    OF_TWIST = 1u << 5,
    OF_BEND = 1u << 6,
    OF_ROUND = 1u << 7,
    OF_ONION = 1u << 8,
    OF_BOUND = 1u << 9,
    OF_NONCONS = 1u << 10,  // ellipsoid / octahedron / hex prism: field can undercut the bounding sphere
    OF_ROT_IDENTITY = 1u << 11,  // rotation exactly the identity (1 on the diagonal, +0 elsewhere)
    OF_ANY_MIRROR = OF_MIRROR_X | OF_MIRROR_Y | OF_MIRROR_Z,
    OF_POINT_OPS = OF_ANY_MIRROR | OF_ELONGATE | OF_REPEAT | OF_TWIST | OF_BEND,
};

// Scene flags
enum : uint32_t {
    SF_SHADOWS = 1u << 0,
    SF_AO = 1u << 1,
    SF_DUAL_SAFE = 1u << 2,
    SF_GI = 1u << 3,
    SF_BLOOM = 1u << 4,
    SF_SECANT = 1u << 5,
};

// 160 bytes. Local point: l = (dot(c0, p - pos), dot(c1, p - pos), dot(c2, p - pos)) * inv,
// where c0..c2 are the rotation's columns (Rᵀ(p - pos) / scale, vec.rs:216-221).
struct alignas(16) DevObject {
    float rot[9];
    float pos[3];
    float inv;    // 1/scale guarded as Transform::to_local
    float scale;
    float params[7];
    uint32_t prim;
    uint32_t mat;
    uint32_t flags;
    uint32_t aux;  // CSG program offset (ops) or volume index
    float k;       // smooth-union radius
    float elongate[3];
    float repeat[3];
    float twist, bend, round, onion;
    float bc[3];   // world bounding sphere (Object::world_bound)
    float br;
};
static_assert(sizeof(DevObject) == 160, "DevObject layout");

enum : uint32_t { SEG_ONE = 0, SEG_RUN = 1, SEG_LINEAR = 2 };
// ONE: a = object index, b = combine.
// RUN: a plain-union run walked as the reference's BVH: ua/ub = its unbounded members in the
//   list `unb`, c = BVH root node (or NIL).
// LINEAR: a plain-union run of at most LINEAR_MAX members that is also folded linearly:
//   a/b = all members (object order) in `unb`; ua/ub/c = the BVH form, used as the exact
//   fallback. A linear fold of every member with the reference's (distance, object index)
//   rule gives the BVH query's result whenever the winner's field is not below its bounding
//   sphere's distance (a subtree the BVH prunes can then never hold the minimum); the only
//   members whose fields can undercut their spheres are exactly-evaluated ellipsoids,
//   octahedra and hexagonal prisms (OF_NONCONS), and a lane whose linear winner is one of those, at a point where
//   its field is not clear of its sphere's bound, re-runs the BVH walk. The linear fold is
//   warp-uniform.
struct alignas(16) DevSegment {
    uint32_t kind, a, b, c;
    uint32_t ua, ub, pad0, pad1;
};
constexpr uint32_t LINEAR_MAX = 48;

struct alignas(16) DevNode {
    float cx, cy, cz, r;
    int32_t left, right, leaf, pad;
};

struct alignas(16) DevMaterial {
    float albedo[3];
    float metallic;
    float specular, roughness, reflectivity;
    float emissive[3];
    uint32_t checker;
    uint32_t pad;
};
static_assert(sizeof(DevMaterial) == 48, "DevMaterial layout");

struct alignas(16) DevLight {
    float vec[3];
    float color[3];
    uint32_t directional;
    float radius;
};

// CSG program op (post-order): PRIM pushes a distance at the current point; XFORM pushes a
// local point; UNXFORM pops it and scales the top distance; binary ops pop two values.
enum : uint32_t {
    CSG_OP_PRIM = 0,
    CSG_OP_XFORM = 1,
    CSG_OP_UNXFORM = 2,
    CSG_OP_UNION = 3,
    CSG_OP_INTERSECT = 4,
    CSG_OP_SUBTRACT = 5,
    CSG_OP_SMOOTH = 6,
    CSG_OP_OFFSET = 7,
    CSG_OP_SHELL = 8,
    CSG_OP_END = 9,
};
struct alignas(16) DevCsgOp {
    uint32_t op, kind, pad0, pad1;
    float p[7];
    float inv;
    float rot[9];
    float pos[3];
    float scale;
    float pad2[3];
};
static_assert(sizeof(DevCsgOp) == 112, "DevCsgOp layout");

struct alignas(16) DevVolume {
    uint32_t nx, ny, nz, valid;
    float min[3], pad0;
    float cell[3], pad1;
    float hi[3], pad2;
    const float* data;  // device address
    uint64_t pad3;
};

struct alignas(16) TapeHeader {
    uint32_t magic, bytes, flags, mode;
    uint32_t n_objects, n_materials, n_lights, n_segments;
    uint32_t n_nodes, n_unbounded, n_csg_ops, n_volumes;
    uint32_t off_objects, off_materials, off_lights, off_segments;
    uint32_t off_nodes, off_unbounded, off_csg, off_volumes;
    uint32_t width, height, aa, bounces;
    // marcher
    uint32_t max_steps, shadow_steps, ao_samples, pad_m;
    float max_dist, eps, step_scale, lod_footprint;
    float subitize, normal_h, slack, fog_density;
    // environment
    float sun_dir[3], pad_e0;
    float ambient[3], pad_e1;
    float sky_ambient[3], pad_e2;
    float fog[3], pad_e3;
    // post
    float exposure, bloom_threshold, bloom_intensity;
    uint32_t bloom_radius;
    // GI ambient cubes: float4 per face, 6 faces per probe, probes (k*ny + j)*nx + i
    float gi_min[3], pad_g0;
    float gi_size[3], pad_g1;
    uint32_t gi_nx, gi_ny, gi_nz, pad_g2;
    const float4* gi_cubes;  // device address
    uint64_t pad_g3;
};

}  // namespace mm3e
