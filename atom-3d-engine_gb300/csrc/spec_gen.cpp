// spec_gen.cpp — the generator of scene-specialised world fields: from a lowered scene tape, the
// CUDA source of its field (objects with their records inlined, CSG programs as straight-line
// code, pre-tests with the scene's constants) and of the march, shadow and AO kernels over it.
// spec.cpp compiles that source with NVRTC and loads the kernels.
#include "spec.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "tape.h"

namespace mm3e {

namespace {
// ---- generator ---------------------------------------------------------------------------------
std::string fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    char b[40];
    std::snprintf(b, sizeof b, "__uint_as_float(0x%08xu)", u);
    return b;
}

std::string farr(const float* f, int n) {
    std::string s = "{";
    for (int i = 0; i < n; ++i) s += (i ? ", " : "") + fbits(f[i]);
    return s + "}";
}

// The initializer of an object record, every float by its bits.
std::string object_rec(const DevObject& o) {
    std::ostringstream os;
    os << "{" << farr(o.rot, 9) << ", " << farr(o.pos, 3) << ", " << fbits(o.inv) << ", " << fbits(o.scale) << ", "
       << farr(o.params, 7) << ", " << o.prim << "u, " << o.mat << "u, " << o.flags << "u, " << o.aux << "u, "
       << fbits(o.k) << ", " << farr(o.elongate, 3) << ", " << farr(o.repeat, 3) << ", " << fbits(o.twist) << ", "
       << fbits(o.bend) << ", " << fbits(o.round) << ", " << fbits(o.onion) << ", " << farr(o.bc, 3) << ", "
       << fbits(o.br) << "}";
    return os.str();
}

// Fields of more objects than this, or with CSG programs, share one out-of-line sincosf for
// their twists and bends (MM3E_SHARED_SINCOS in device_math.cuh). Measured: the specialised
// frames of 16 seeded procedural scenes (8-64 primitives, CSG trees, domain ops; 256^2 to 1080p)
// 3.23x faster than the interpreter's (time-weighted) with it, 2.84x without; the feature gallery
// (15 objects, whose march is not fetch-bound) 3.6% slower with it.
constexpr uint32_t kSharedSincosObjects = 16;

// Fields of more objects than this take no weak bound for CSG objects and no weak skip of
// unbounded one-object segments: their tests run at every sample, and in a field that large the
// code they add costs more in instruction fetch than the exact evaluations they save.
constexpr uint32_t kWeakExtraObjects = 32;

// A CSG program (csg.rs:95-118, the post-order stack program csg_eval runs over `op`, at most
// `n` ops) as straight-line code over the local point `l`: the stack depths after every op are
// known when the program is generated, so each stack slot becomes a named local and each
// primitive and transform gets its constants inline. Every arithmetic step is the interpreter's,
// in its order. Empty when the program is not one the interpreter runs to a well-defined end
// (a stack underflow or overflow); the object then keeps the interpreter.
std::string csg_body(const DevCsgOp* op, size_t n) {
    std::ostringstream os;
    std::vector<std::string> vals, pts;
    std::string cur = "l";
    int nv = 0, np = 0;
    for (size_t g = 0; g < 4096 && g < n; ++g, ++op) {
        const uint32_t o = op->op;
        if (o == CSG_OP_PRIM) {
            if (vals.size() >= (size_t)MAX_CSG_STACK) return "";
            const std::string q = "q" + std::to_string(nv), v = "v" + std::to_string(nv);
            os << "    const float " << q << "[7] = " << farr(op->p, 7) << ";\n    float " << v
               << " = prim_distance(" << op->kind << "u, " << q << ", " << cur << ");\n";
            nv += 1;
            vals.push_back(v);
        } else if (o == CSG_OP_XFORM) {
            if (pts.size() >= (size_t)MAX_CSG_STACK) return "";
            const std::string r = "r" + std::to_string(np), x = "x" + std::to_string(np);
            os << "    const float " << r << "[9] = " << farr(op->rot, 9) << ";\n    const V " << x << " = scale(rot_t("
               << r << ", " << cur << " - V{" << fbits(op->pos[0]) << ", " << fbits(op->pos[1]) << ", "
               << fbits(op->pos[2]) << "}), " << fbits(op->inv) << ");\n";
            np += 1;
            pts.push_back(cur);
            cur = x;
        } else if (o == CSG_OP_UNXFORM) {
            if (pts.empty() || vals.empty()) return "";
            cur = pts.back();
            pts.pop_back();
            os << "    " << vals.back() << " = " << vals.back() << " * " << fbits(op->scale) << ";\n";
        } else if (o == CSG_OP_UNION || o == CSG_OP_INTERSECT || o == CSG_OP_SUBTRACT || o == CSG_OP_SMOOTH) {
            if (vals.size() < 2) return "";
            const std::string b = vals.back();
            vals.pop_back();
            const std::string a = vals.back();
            if (o == CSG_OP_UNION) os << "    " << a << " = fminf(" << a << ", " << b << ");\n";
            if (o == CSG_OP_INTERSECT) os << "    " << a << " = fmaxf(" << a << ", " << b << ");\n";
            if (o == CSG_OP_SUBTRACT) os << "    " << a << " = fmaxf(" << a << ", -" << b << ");\n";
            if (o == CSG_OP_SMOOTH)
                os << "    " << a << " = f_smooth_union(Field{" << a << ", 0u}, Field{" << b << ", 0u}, "
                   << fbits(op->p[0]) << ").d;\n";
        } else if (o == CSG_OP_OFFSET || o == CSG_OP_SHELL) {
            if (vals.empty()) return "";
            const std::string a = vals.back();
            if (o == CSG_OP_OFFSET) os << "    " << a << " = " << a << " - " << fbits(op->p[0]) << ";\n";
            else os << "    " << a << " = fabsf(" << a << ") - " << fbits(op->p[0]) << ";\n";
        } else {
            break;
        }
    }
    os << "    return " << (vals.empty() ? std::string("__int_as_float(0x7f800000)") : vals.front()) << ";\n";
    return os.str();
}

// A plane whose normal is an axis, (+-1 on axis k, +0 on the others), with the identity
// rotation, no point operations and an offset other than -0. For a finite local point l its
// field dot(l, n) + h = ((l.x n.x + l.y n.y) + l.z n.z) + h is fl(+-l_k + h) bit for bit: the
// products by +0 are zeros, which leave a nonzero sum as it is; where +-l_k is itself zero the
// sum is a zero, and adding h gives h (h != 0) or +0 (h = +0) whatever the zeros' signs. For the
// same reason the sign fix-ups of the identity rotation cannot show, so l_k is (p_k - pos_k) inv.
bool axis_plane(const DevObject& o, int& k, bool& neg) {
    if (o.prim != 10u || !(o.flags & OF_ROT_IDENTITY) || (o.flags & OF_POINT_OPS)) return false;
    if (!std::isfinite(o.inv) || o.inv == 0.0f) return false;
    uint32_t bits[4];
    std::memcpy(bits, o.params, sizeof bits);
    if (bits[3] == 0x80000000u || !std::isfinite(o.params[3])) return false;
    k = -1;
    for (int a = 0; a < 3; ++a) {
        if (bits[a] == 0x3f800000u || bits[a] == 0xbf800000u) {
            if (k >= 0) return false;
            k = a;
            neg = bits[a] == 0xbf800000u;
        } else if (bits[a] != 0u) {
            return false;
        }
    }
    return k >= 0;
}

// An object's field with its record inlined; a CSG object's program is generated code too
// (csg_ops: the tape's CSG ops, n_csg of them), and an axis-aligned plane is one addition.
std::string object_fn(uint32_t i, const DevObject& o, const DevCsgOp* csg_ops, uint32_t n_csg) {
    std::ostringstream os;
    const std::string body = o.prim == 11u && o.aux < n_csg ? csg_body(csg_ops + o.aux, n_csg - o.aux) : "";
    if (!body.empty())
        os << "__device__ __forceinline__ float csg_" << i << "(V l) {\n" << body << "}\n";
    os << "__device__ __forceinline__ Field obj_" << i << "(const Tape& T, V p) {\n"
       << "    const DevObject o = " << object_rec(o) << ";\n";
    int k = -1;
    bool neg = false;
    if (!body.empty()) {
        os << "    return object_finish(o, csg_" << i << "(local_point(o, p)));\n}\n";
    } else if (axis_plane(o, k, neg)) {
        const char* axis[3] = {"p.x", "p.y", "p.z"};
        os << "    const float lk = (" << axis[k] << " - " << fbits(o.pos[k]) << ") * " << fbits(o.inv) << ";\n"
           << "    return object_finish(o, " << (neg ? "-lk" : "lk") << " + " << fbits(o.params[3]) << ");  // axis plane\n}\n";
    } else {
        os << "    return object_field(T, o, p);\n}\n";
    }
    return os.str();
}

// Leaves (object indices) of the BVH below node `root`.
void bvh_leaves(const DevNode* node, uint32_t n_nodes, uint32_t root, std::vector<uint32_t>& out) {
    if (root == NIL || root >= n_nodes) return;
    std::vector<uint32_t> todo{root};
    while (!todo.empty()) {
        uint32_t k = todo.back();
        todo.pop_back();
        const DevNode& nd = node[k];
        if (nd.leaf >= 0) {
            out.push_back((uint32_t)nd.leaf);
            continue;
        }
        if (nd.left >= 0 && (uint32_t)nd.left < n_nodes) todo.push_back((uint32_t)nd.left);
        if (nd.right >= 0 && (uint32_t)nd.right < n_nodes) todo.push_back((uint32_t)nd.right);
    }
    std::sort(out.begin(), out.end());
}

// A plain-union run's Bvh::query (accel.rs:79-119) as generated code: bvh_segment's steps (its
// unbounded members exactly in list order, then the sphere BVH near child first with the
// `lower > best` prune and the `lower > slack` substitute, (distance, lowest index) fold), with
// the run's objects dispatched to their inlined fields. Inlined at its call site, so the
// specialised kernels make no function call (a call there costs a stack frame and spills).
std::string walk_fn(uint32_t s, const DevSegment& sg, const DevNode* node, uint32_t n_nodes, const uint32_t* unb,
                    float slack, bool seeded) {
    std::ostringstream os;
    os << "__device__ __forceinline__ Field walk_" << s << "(const Tape& T, V p, Field acc) {\n"
       << "    const float INF = __int_as_float(0x7f800000);\n"
       << "    float bd = " << (seeded ? "acc.d" : "INF") << ";\n    int32_t bi = " << (seeded ? "-1" : "0x7FFFFFFF")
       << ";\n    uint32_t bm = " << (seeded ? "acc.m" : "0u") << ";\n";
    for (uint32_t u = sg.ua; u < sg.ua + sg.ub; ++u)
        os << "    {\n        Field f = obj_" << unb[u] << "(T, p);\n        if (f.d < bd || (f.d == bd && " << unb[u]
           << " < bi)) {\n            bd = f.d;\n            bi = " << unb[u] << ";\n            bm = f.m;\n        }\n    }\n";
    std::vector<uint32_t> leaves;
    bvh_leaves(node, n_nodes, sg.c, leaves);
    if (!leaves.empty()) {
        os << "    NodeStack stk;\n    stk.clear();\n    stk.push(" << sg.c << "u);\n"
           << "    while (stk.n > 0) {\n"
           << "        const DevNode& nd = T.node[stk.pop()];\n"
           << "        const float nd2 = length_sq(p - V{nd.cx, nd.cy, nd.cz});\n"
           << "        if (far_beyond(nd2, bd, nd.r)) continue;\n"
           << "        const float lower = sqrtf(nd2) - nd.r;\n"
           << "        if (lower > bd) continue;\n"
           << "        if (nd.leaf >= 0) {\n"
           << "            const int32_t i = nd.leaf;\n"
           << "            if (lower > " << fbits(slack) << ") {\n"
           << "                if (lower < bd || (lower == bd && i < bi)) {\n"
           << "                    bd = lower;\n                    bi = i;\n                    bm = T.obj[i].mat;\n"
           << "                }\n                continue;\n            }\n"
           << "            Field f;\n            switch (i) {\n";
        for (uint32_t i : leaves) os << "                case " << i << ": f = obj_" << i << "(T, p); break;\n";
        os << "                default: f = Field{INF, 0u}; break;\n            }\n"
           << "            if (f.d < bd || (f.d == bd && i < bi)) {\n"
           << "                bd = f.d;\n                bi = i;\n                bm = f.m;\n            }\n"
           << "            continue;\n        }\n"
           << "        const DevNode& L = T.node[nd.left];\n        const DevNode& R = T.node[nd.right];\n"
           << "        const float ld = length_sq(p - V{L.cx, L.cy, L.cz});\n"
           << "        const float rd = length_sq(p - V{R.cx, R.cy, R.cz});\n"
           << "        const bool lnear = ld <= rd;\n"
           << "        stk.push(lnear ? (uint32_t)nd.right : (uint32_t)nd.left);\n"
           << "        stk.push(lnear ? (uint32_t)nd.left : (uint32_t)nd.right);\n"
           << "    }\n";
    }
    os << "    return Field{bd, bm};\n}\n";
    return os.str();
}

// A lower bound of an object's field that holds wherever it is positive: with l the local point
// (rotation and 1/scale applied; before mirror, elongate, repeat, twist and bend),
//   field(p) >= c * (n - R) * scale - post,   n = |l| over the axes that do not repeat,
// because mirror, twist and bend preserve |l|, elongate by h moves it by at most |h| (added to
// R), a periodic axis can only lower the norm the primitive sees, and each primitive's field is
// at least c * (|q| - R) outside the ball of radius R about its local origin: c = 1 for the
// exact distances, 0.577 for the octahedron's bound field ((|x|+|y|+|z| - s) * 0.5773503 with
// |x|+|y|+|z| >= |q|), r_min / r_max for the ellipsoid's (k0 (k0 - 1) / k1 with k1 <= k0 / r_min
// and k0 >= |q| / r_max). post = round (any sign) + onion (>= 0 only).
struct WeakBound {
    bool ok = false;
    float R = 0.0f, c = 0.0f, post = 0.0f;
    bool axis[3] = {true, true, true};
};

// A primitive's weak constants: its field is at least c * (|q| - R) outside the ball of radius R
// about its local origin (see WeakBound). False for a plane (unbounded) and unknown kinds.
bool prim_weak(uint32_t kind, const float* q, double& R, double& c) {
    c = 0.999;
    switch (kind) {
        case 0: R = q[0]; break;
        case 1:
        case 2: R = std::sqrt((double)q[0] * q[0] + (double)q[1] * q[1] + (double)q[2] * q[2]); break;
        case 3: R = (double)q[0] + q[1]; break;
        case 4: R = std::sqrt((double)q[0] * q[0] + (double)q[1] * q[1]); break;
        case 5: {
            double a = std::sqrt((double)q[0] * q[0] + (double)q[1] * q[1] + (double)q[2] * q[2]);
            double b = std::sqrt((double)q[3] * q[3] + (double)q[4] * q[4] + (double)q[5] * q[5]);
            R = std::max(a, b) + q[6];
            break;
        }
        case 6: R = std::max((double)q[0], (double)q[2] + q[1]); break;
        case 7: {
            double rmax = std::max(std::max(q[0], q[1]), q[2]), rmin = std::min(std::min(q[0], q[1]), q[2]);
            if (!(rmin > 0.0)) return false;
            R = rmax;
            c = 0.999 * rmin / rmax;
            break;
        }
        case 8: R = q[0]; c = 0.577; break;
        case 9: {
            double circ = 2.0 * q[0] / std::sqrt(3.0);
            R = std::sqrt(circ * circ + (double)q[1] * q[1]);
            break;
        }
        default: return false;  // plane, CSG, volume
    }
    return R >= 0.0 && std::isfinite(R);
}

// A CSG program's weak constants (csg.rs:95-118; the post-order program csg_eval runs), from the
// bounds of its parts: with each part's field at least c_i (|q| - R_i) - post_i outside its ball,
//   union, smooth union:  min over the parts, so c = min c_i, R = max R_i, post = max post_i
//                         (+ k/4 for the smooth one, whose blend is at least the minimum - k/4);
//   intersection:         at least either part (the one with the smaller ball is kept);
//   subtraction:          at least its first part;
//   offset o, shell t:    post + o, post + t (|d| - t >= d - t);
//   transform (pos, s):   the part at the local point R^T (q - pos) / s, times s: c kept, R =
//                         |pos| + s R_part, post = s post_part (the rotation keeps norms, checked).
// False when a part has no bound (a plane) or the program is not one the interpreter runs to a
// defined end.
bool csg_weak(const DevCsgOp* op, size_t n, double& R, double& c, double& post) {
    struct Part {
        double R, c, post;
    };
    std::vector<Part> vals;
    std::vector<double> pos_norm;
    for (size_t g = 0; g < 4096 && g < n; ++g, ++op) {
        const uint32_t k = op->op;
        if (k == CSG_OP_PRIM) {
            Part pt{0.0, 0.0, 0.0};
            if (!prim_weak(op->kind, op->p, pt.R, pt.c)) return false;
            vals.push_back(pt);
        } else if (k == CSG_OP_XFORM) {
            const float* r = op->rot;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double d = (double)r[a * 3] * r[b * 3] + (double)r[a * 3 + 1] * r[b * 3 + 1] +
                               (double)r[a * 3 + 2] * r[b * 3 + 2];
                    if (std::fabs(d - (a == b ? 1.0 : 0.0)) > 1e-5) return false;
                }
            pos_norm.push_back(std::sqrt((double)op->pos[0] * op->pos[0] + (double)op->pos[1] * op->pos[1] +
                                         (double)op->pos[2] * op->pos[2]));
        } else if (k == CSG_OP_UNXFORM) {
            if (vals.empty() || pos_norm.empty() || !(op->scale > 0.0f)) return false;
            Part& t = vals.back();
            t.R = pos_norm.back() + (double)op->scale * t.R;
            t.post = (double)op->scale * t.post;
            pos_norm.pop_back();
        } else if (k == CSG_OP_UNION || k == CSG_OP_SMOOTH || k == CSG_OP_INTERSECT || k == CSG_OP_SUBTRACT) {
            if (vals.size() < 2) return false;
            const Part b = vals.back();
            vals.pop_back();
            Part& a = vals.back();
            if (k == CSG_OP_UNION || k == CSG_OP_SMOOTH) {
                a = Part{std::max(a.R, b.R), std::min(a.c, b.c), std::max(a.post, b.post)};
                if (k == CSG_OP_SMOOTH && op->p[0] > 0.0f) a.post += 0.25 * (double)op->p[0];
            } else if (k == CSG_OP_INTERSECT && b.R < a.R) {
                a = b;
            }
        } else if (k == CSG_OP_OFFSET || k == CSG_OP_SHELL) {
            if (vals.empty()) return false;
            vals.back().post += (double)op->p[0];
        } else {
            break;
        }
    }
    if (vals.size() != 1 || !pos_norm.empty()) return false;
    R = vals[0].R;
    c = vals[0].c;
    post = vals[0].post;
    return R >= 0.0 && std::isfinite(R) && std::isfinite(post) && c > 0.0;
}

WeakBound weak_bound(const DevObject& o, const DevCsgOp* csg, uint32_t n_csg) {
    WeakBound w;
    double R = 0.0, c = 0.999, shape_post = 0.0;
    if (o.prim == 11u) {
        if (!csg || o.aux >= n_csg || !csg_weak(csg + o.aux, n_csg - o.aux, R, c, shape_post)) return w;
    } else if (!prim_weak(o.prim, o.params, R, c)) {
        return w;
    }
    if (!(R >= 0.0) || !std::isfinite(R)) return w;
    if (o.flags & OF_ELONGATE)
        R += std::sqrt((double)o.elongate[0] * o.elongate[0] + (double)o.elongate[1] * o.elongate[1] +
                       (double)o.elongate[2] * o.elongate[2]);
    int kept = 3;
    if (o.flags & OF_REPEAT)
        for (int a = 0; a < 3; ++a)
            if (o.repeat[a] > 0.0f) {
                w.axis[a] = false;
                kept -= 1;
            }
    if (kept == 0) return w;
    double post = shape_post * (double)o.scale;
    if (o.flags & OF_ROUND) post += o.round;
    if (o.flags & OF_ONION) {
        if (!(o.onion >= 0.0f)) return w;
        post += o.onion;
    }
    R = R * (1.0 + 1.0 / 4096.0) + 1e-6;
    w.R = (float)R;
    w.c = (float)c;
    w.post = (float)(post + std::fabs(post) / 4096.0 + 1e-6);
    w.ok = std::isfinite(w.R) && std::isfinite(w.post) && o.scale > 0.0f;
    return w;
}

// The nearest binary32 value at or below x.
float float_at_or_below(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -std::numeric_limits<float>::infinity());
    return f;
}

// The nearest binary32 value at or above x.
float float_at_or_above(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

// The weak-bound cull of a member: true when its field cannot reach down to bd.
// The bound only takes the norm of the local point, so an identity rotation is left out (the
// skipped products could only change the signs of zero coordinates). With positive constants the
// test compares squared norms (weak_beyond_sq); a trailing comment keeps the bound's R, c, scale
// and post for the soundness tests.
std::string weak_cull_expr(const DevObject& o, const WeakBound& w, const std::string& thr = "bd") {
    std::ostringstream os;
    const std::string d =
        "p - V{" + fbits(o.pos[0]) + ", " + fbits(o.pos[1]) + ", " + fbits(o.pos[2]) + "}";
    const std::string local = "scale(" + ((o.flags & OF_ROT_IDENTITY) ? d : "rot_t_fma(RO, " + d + ")") + ", " +
                              fbits(o.inv) + "), " + (w.axis[0] ? "true" : "false") + ", " +
                              (w.axis[1] ? "true" : "false") + ", " + (w.axis[2] ? "true" : "false");
    const double eps = 1.0 / 1024.0;
    const double K = (double)o.scale * ((double)w.c - eps);
    const double A = (double)w.post + (double)w.R * (double)o.scale * ((double)w.c + eps);
    const float Af = float_at_or_above(A), Bf = float_at_or_above((1.0 + 1.0 / 131072.0) / K);
    if (K > 0.0 && A > 0.0 && std::isfinite(Af) && std::isfinite(Bf)) {
        os << "weak_beyond_sq(" << local << ", " << fbits(Af) << ", " << fbits(Bf) << ", " << thr << ") /* weak bound R c scale post: "
           << fbits(w.R) << " " << fbits(w.c) << " " << fbits(o.scale) << " " << fbits(w.post) << " */";
    } else {
        os << "weak_beyond(" << local << ", " << fbits(w.R) << ", " << fbits(w.c) << ", " << fbits(o.scale) << ", "
           << fbits(w.post) << ", " << thr << ")";
    }
    return os.str();
}

// A sphere with the identity rotation, unit scale and no modifiers whose bounding sphere is
// itself: its exact field, length(p - pos) - r (the identity rotation only changes the signs of
// zero coordinates, which the squares drop), equals the bound distance sqrtf(|p - c|^2) - r bit for
// bit, so a member needs no second evaluation.
bool plain_sphere(const DevObject& o) {
    return o.prim == 0u && (o.flags & OF_BOUND) && (o.flags & OF_ROT_IDENTITY) &&
           !(o.flags & (OF_POINT_OPS | OF_ROUND | OF_ONION)) && o.scale == 1.0f && o.inv == 1.0f &&
           o.bc[0] == o.pos[0] && o.bc[1] == o.pos[1] && o.bc[2] == o.pos[2] && o.br == o.params[0];
}

// The linearised sphere pre-test (far_beyond_lin in device_math.cuh) of the sphere (c, r)
// against `thr`, which `pos` marks as never negative; CB is the evaluation's cull_base(p). The
// constants are -2c (exact), mu |c|^2 rounded down, 2 M r and M r^2 rounded up (mu = 1 - 2^-19,
// M = 1 + 2^-14), each from binary64 arithmetic nudged by 2^-50 the safe way. Empty when the
// sphere's radius is not a finite non-negative number.
std::string lin_test(const float* c, float r, const std::string& thr, bool pos) {
    if (!(r >= 0.0f) || !std::isfinite(r)) return "";
    const double mu = 1.0 - std::ldexp(1.0, -19), M = 1.0 + std::ldexp(1.0, -14), nudge = std::ldexp(1.0, -50);
    const double cc = (double)c[0] * c[0] + (double)c[1] * c[1] + (double)c[2] * c[2];
    const float c2 = float_at_or_below(mu * cc * (1.0 - nudge));
    const float m2r = float_at_or_above(2.0 * M * (double)r * (1.0 + nudge));
    const float mr2 = float_at_or_above(M * (double)r * (double)r * (1.0 + nudge));
    if (!std::isfinite(c2) || !std::isfinite(m2r) || !std::isfinite(mr2)) return "";
    return std::string(pos ? "far_beyond_lin_pos" : "far_beyond_lin") + "(dist2_below(p, CB, " + fbits(-2.0f * c[0]) +
           ", " + fbits(-2.0f * c[1]) + ", " + fbits(-2.0f * c[2]) + ", " + fbits(c2) + "), " + thr + ", " + fbits(m2r) +
           ", " + fbits(mr2) + ")";
}

std::string lower_expr(const DevObject& o) {
    return "length(p - V{" + fbits(o.bc[0]) + ", " + fbits(o.bc[1]) + ", " + fbits(o.bc[2]) + "}) - " + fbits(o.br);
}

// Spatial groups of at most 4 union members (median splits on the longest axis of their bound
// centres) with an enclosing sphere: for every member, |c - ci| + ri <= r holds in exact
// arithmetic with a relative margin of 2^-20, so a member's own bound test never keeps a point
// that the cluster's test culled.
struct MemberCluster {
    std::vector<uint32_t> members;
    float c[3];
    float r;
};

void cluster_members(const DevObject* obj, std::vector<uint32_t> m, std::vector<MemberCluster>& out) {
    if (m.empty()) return;
    if (m.size() <= 4) {
        MemberCluster cl;
        cl.members = m;
        double mean[3] = {0.0, 0.0, 0.0};
        for (uint32_t i : m)
            for (int a = 0; a < 3; ++a) mean[a] += obj[i].bc[a];
        for (int a = 0; a < 3; ++a) cl.c[a] = (float)(mean[a] / (double)m.size());
        double r = 0.0;
        for (uint32_t i : m) {
            double dx = (double)obj[i].bc[0] - cl.c[0], dy = (double)obj[i].bc[1] - cl.c[1],
                   dz = (double)obj[i].bc[2] - cl.c[2];
            double e = std::sqrt(dx * dx + dy * dy + dz * dz) + (double)obj[i].br;
            if (e > r) r = e;
        }
        r = r * (1.0 + 1.0 / 1048576.0) + 1e-30;
        float rf = (float)r;
        if ((double)rf < r) rf = std::nextafter(rf, INFINITY);
        cl.r = rf;
        out.push_back(std::move(cl));
        return;
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i : m)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], obj[i].bc[a]);
            hi[a] = std::max(hi[a], obj[i].bc[a]);
        }
    int axis = 0;
    for (int a = 1; a < 3; ++a)
        if (hi[a] - lo[a] > hi[axis] - lo[axis]) axis = a;
    std::stable_sort(m.begin(), m.end(), [&](uint32_t x, uint32_t y) { return obj[x].bc[axis] < obj[y].bc[axis]; });
    size_t half = m.size() / 2;
    cluster_members(obj, std::vector<uint32_t>(m.begin(), m.begin() + half), out);
    cluster_members(obj, std::vector<uint32_t>(m.begin() + half, m.end()), out);
}

// A sphere enclosing the given spheres: |c - c_i| + r_i <= r for each of them in exact
// arithmetic with a relative margin of 2^-20 (the same rule as the clusters' spheres).
bool enclosing_sphere(const std::vector<std::pair<const float*, float>>& spheres, float* c, float& r) {
    double mean[3] = {0.0, 0.0, 0.0};
    for (const auto& sp : spheres)
        for (int a = 0; a < 3; ++a) mean[a] += sp.first[a];
    for (int a = 0; a < 3; ++a) c[a] = (float)(mean[a] / (double)spheres.size());
    double rr = 0.0;
    for (const auto& sp : spheres) {
        if (!(sp.second >= 0.0f) || !std::isfinite(sp.second)) return false;
        double dx = (double)sp.first[0] - c[0], dy = (double)sp.first[1] - c[1], dz = (double)sp.first[2] - c[2];
        rr = std::max(rr, std::sqrt(dx * dx + dy * dy + dz * dz) + (double)sp.second);
    }
    rr = rr * (1.0 + 1.0 / 1048576.0) + 1e-30;
    float rf = (float)rr;
    if ((double)rf < rr) rf = std::nextafter(rf, INFINITY);
    r = rf;
    return std::isfinite(r) && std::isfinite(c[0]) && std::isfinite(c[1]) && std::isfinite(c[2]);
}

}  // namespace

SpecSize spec_size(const std::vector<unsigned char>& blob) {
    const TapeHeader* h = reinterpret_cast<const TapeHeader*>(blob.data());
    const DevObject* obj = reinterpret_cast<const DevObject*>(blob.data() + h->off_objects);
    const DevSegment* seg = reinterpret_cast<const DevSegment*>(blob.data() + h->off_segments);
    const uint32_t* unb = reinterpret_cast<const uint32_t*>(blob.data() + h->off_unbounded);
    const DevCsgOp* csg = reinterpret_cast<const DevCsgOp*>(blob.data() + h->off_csg);
    SpecSize z;
    auto count = [&](uint32_t i) {
        z.objects += 1;
        if (obj[i].prim == 11u)
            for (const DevCsgOp* op = csg + obj[i].aux; op->op != CSG_OP_END && z.csg_ops < (1u << 20); ++op)
                z.csg_ops += 1;
    };
    for (uint32_t s = 0; s < h->n_segments; ++s) {
        if (seg[s].kind == SEG_ONE) count(seg[s].a);
        if (seg[s].kind == SEG_LINEAR)
            for (uint32_t k = 0; k < seg[s].b; ++k) count(unb[seg[s].a + k]);
    }
    return z;
}

std::string spec_source(const std::vector<unsigned char>& blob, uint32_t block, uint32_t unroll, bool smem_tape,
                        uint32_t min_blocks) {
    const TapeHeader* h = reinterpret_cast<const TapeHeader*>(blob.data());
    const DevObject* obj = reinterpret_cast<const DevObject*>(blob.data() + h->off_objects);
    const DevSegment* seg = reinterpret_cast<const DevSegment*>(blob.data() + h->off_segments);
    const uint32_t* unb = reinterpret_cast<const uint32_t*>(blob.data() + h->off_unbounded);
    std::ostringstream os;
    os << "// scene-specialised world field (generated)\n"
          "typedef unsigned int uint32_t;\ntypedef int int32_t;\ntypedef unsigned long long uint64_t;\n"
          "typedef unsigned short uint16_t;\ntypedef unsigned char uint8_t;\ntypedef long long int64_t;\n"
       << (h->n_objects > kSharedSincosObjects || h->n_csg_ops > 0 ? "#define MM3E_SHARED_SINCOS 1\n" : "")
       << "#include \"march_kernels.cuh\"\n"
          "namespace mm3e {\nnamespace spec {\n";
    const DevNode* node = reinterpret_cast<const DevNode*>(blob.data() + h->off_nodes);
    // segments that need the BVH walk: big runs, and LINEAR runs with a non-conservative member
    // (whose winner may undercut its sphere)
    std::vector<bool> walk(h->n_segments, false);
    for (uint32_t s = 0; s < h->n_segments; ++s) {
        const DevSegment& sg = seg[s];
        if (sg.kind == SEG_RUN) walk[s] = true;
        if (sg.kind == SEG_LINEAR)
            for (uint32_t k = 0; k < sg.b; ++k) {
                const DevObject& o = obj[unb[sg.a + k]];
                if ((o.flags & OF_NONCONS) && (o.flags & OF_BOUND)) walk[s] = true;
            }
    }
    std::vector<bool> used(h->n_objects, false);
    for (uint32_t s = 0; s < h->n_segments; ++s) {
        const DevSegment& sg = seg[s];
        if (sg.kind == SEG_ONE) used[sg.a] = true;
        if (sg.kind == SEG_LINEAR)
            for (uint32_t k = 0; k < sg.b; ++k) used[unb[sg.a + k]] = true;
        if (walk[s]) {
            for (uint32_t u = sg.ua; u < sg.ua + sg.ub; ++u) used[unb[u]] = true;
            std::vector<uint32_t> leaves;
            bvh_leaves(node, h->n_nodes, sg.c, leaves);
            for (uint32_t i : leaves)
                if (i < h->n_objects) used[i] = true;
        }
    }
    const DevCsgOp* csg = reinterpret_cast<const DevCsgOp*>(blob.data() + h->off_csg);
    for (uint32_t i = 0; i < h->n_objects; ++i)
        if (used[i]) os << object_fn(i, obj[i], csg, h->n_csg_ops);
    for (uint32_t s = 0; s < h->n_segments; ++s)
        if (walk[s]) os << walk_fn(s, seg[s], node, h->n_nodes, unb, h->slack, s > 0);
    const std::string slack = fbits(h->slack);
    const bool weak_extra = h->n_objects <= kWeakExtraObjects;
    const DevCsgOp* weak_csg = weak_extra ? csg : nullptr;  // CSG objects get weak bounds only then
    // pre-tests against fmaxf(x, slack) need no sign test of the threshold when slack > 0
    const bool slack_pos = h->slack > 0.0f;
    const std::string fb_pos = slack_pos ? "far_beyond_pos" : "far_beyond";
    // a sphere pre-test: the linearised form, or the squared distance where that is not available
    auto sphere_test = [&](const float* c, float r, const std::string& thr, bool pos) -> std::string {
        const std::string lt = lin_test(c, r, thr, pos);
        if (!lt.empty()) return lt;
        return std::string(pos ? fb_pos : std::string("far_beyond")) + "(length_sq_fma(p - V{" + fbits(c[0]) + ", " +
               fbits(c[1]) + ", " + fbits(c[2]) + "}), " + thr + ", " + fbits(r) + ")";
    };
    os << "__device__ __forceinline__ Field eval(const Tape& T, V p) {\n"
          "    const float INF = __int_as_float(0x7f800000);\n"
          "    const float CB = cull_base(p);\n"
          "    Field acc{INF, 0u};\n";
    for (uint32_t s = 0; s < h->n_segments; ++s) {
        const DevSegment& sg = seg[s];
        const bool seeded = s > 0;
        os << "    {  // segment " << s << "\n";
        if (sg.kind == SEG_ONE) {
            const DevObject& o = obj[sg.a];
            // A bounded object whose sphere distance clears the slack and a threshold set by the
            // accumulated field leaves the accumulator as it is (one_keeps_acc in device_math.cuh:
            // the accumulator for a union, the accumulator plus k rounded up for a smooth union,
            // whose blend weight is then exactly 1, minus the accumulator for a subtraction): the
            // squared pre-test skips the segment there. Never for an accumulator that is not
            // finite, nor a zero one under a smooth union.
            const bool smooth = sg.b == 1u && o.k > 0.0f;
            const bool skip = seeded && (o.flags & OF_BOUND) && sg.b <= 2u;
            if (skip) {
                const std::string thr = smooth      ? "__fadd_ru(acc.d, " + fbits(o.k) + ")"
                                        : sg.b == 2u ? std::string("-acc.d")
                                                     : std::string("acc.d");
                const std::string keep = "fabsf(acc.d) < INF" + std::string(smooth ? " && acc.d != 0.0f" : "");
                const std::string thr2 = "fmaxf(" + thr + ", " + slack + ")";
                const std::string lt = lin_test(o.bc, o.br, thr2, slack_pos);
                if (!lt.empty())
                    os << "        if (!(" << keep << " && " << lt << ")) {\n";
                else
                    os << "        if (!(" << keep << " && " << fb_pos << "(length_sq_fma(p - V{" << fbits(o.bc[0]) << ", "
                       << fbits(o.bc[1]) << ", " << fbits(o.bc[2]) << "}), " << thr2 << ", " << fbits(o.br) << "))) {\n";
            }
            // An unbounded object with a weak bound (bend, repeat; CSG programs) skips the same way
            // where that bound clears the threshold: no bound substitute stands in for its field,
            // so the threshold is the accumulator's alone.
            const bool weak_skip = weak_extra && seeded && !(o.flags & OF_BOUND) && sg.b <= 2u;
            const WeakBound owb = weak_skip ? weak_bound(o, weak_csg, h->n_csg_ops) : WeakBound{};
            if (owb.ok) {
                const std::string thr = smooth      ? "__fadd_ru(acc.d, " + fbits(o.k) + ")"
                                        : sg.b == 2u ? std::string("-acc.d")
                                                     : std::string("acc.d");
                if (!(o.flags & OF_ROT_IDENTITY)) os << "        const float RO[9] = " << farr(o.rot, 9) << ";\n";
                os << "        if (!(fabsf(acc.d) < INF" << (smooth ? " && acc.d != 0.0f" : "") << " && "
                   << weak_cull_expr(o, owb, thr) << ")) {  // weak skip\n";
            }
            os << "        Field f;\n        bool sub = false;\n";
            if (o.flags & OF_BOUND)
                os << "        {\n            float lower = " << lower_expr(o) << ";\n"
                   << "            if (lower > " << slack << ") {\n                f = Field{lower, " << o.mat
                   << "u};\n                sub = true;\n            }\n        }\n";
            os << "        if (!sub) f = obj_" << sg.a << "(T, p);\n";
            // the bound substitute folds with the segment's combine, the exact field with the
            // object's own (the same value; both kept as the interpreter has them)
            uint32_t comb_exact = (o.flags >> 16) & 3u;
            auto fold = [&](uint32_t comb) -> std::string {
                if (!seeded) return "acc = f;";
                if (comb == 0u) return "acc = f_union(acc, f);";
                if (comb == 1u) return "acc = f_smooth_union(acc, f, " + fbits(o.k) + ");";
                return "acc = f_subtract(acc, f);";
            };
            if (comb_exact == sg.b) os << "        " << fold(sg.b) << "\n";
            else os << "        if (sub) { " << fold(sg.b) << " } else { " << fold(comb_exact) << " }\n";
            if (skip || owb.ok) os << "        }\n";
        } else if (sg.kind == SEG_LINEAR) {
            // The fold is an argmin with lowest-index ties (the seed, index -1, wins its ties), and
            // a culled member cannot reach the minimum, so any member order gives the same
            // result: members that are never culled go first, then the cullable ones in spatial
            // clusters whose enclosing-sphere pre-test skips a whole cluster at once.
            bool any_noncons = false;
            os << "        float bd = " << (seeded ? "acc.d" : "INF") << ";\n        int32_t bi = "
               << (seeded ? "-1" : "0x7FFFFFFF") << ";\n        uint32_t bm = " << (seeded ? "acc.m" : "0u")
               << ";\n        bool bnc = false;\n";
            std::vector<uint32_t> cullable;
            auto member = [&](uint32_t i, bool cull) {
                const DevObject& o = obj[i];
                if (cull && plain_sphere(o)) {
                    os << "        {  // member " << i << " (its exact field is its bound distance)\n"
                       << "            if (!" << sphere_test(o.bc, o.br, "bd", false) << ") {\n"
                       << "            const float lower = " << lower_expr(o) << ";\n"
                       << "            if (lower < bd || (lower == bd && " << i << " < bi)) {\n                bd = lower;\n"
                       << "                bi = " << i << ";\n                bm = " << o.mat
                       << "u;\n                bnc = false;\n            }\n            }\n        }\n";
                    return;
                }
                bool nc = (o.flags & OF_NONCONS) != 0;
                // a bounded OF_NONCONS winner needs the BVH walk only where it may undercut its sphere
                const bool nc_bounded = nc && (o.flags & OF_BOUND);
                const std::string undercut = nc_bounded ? "noncons_undercut(f.d, lower, " + fbits(o.br) + ")" : "false";
                std::string exact = "Field f = obj_" + std::to_string(i) + "(T, p);\n            if (f.d < bd || (f.d == bd && " +
                                    std::to_string(i) + " < bi)) {\n                bd = f.d;\n                bi = " +
                                    std::to_string(i) + ";\n                bm = f.m;\n                bnc = " +
                                    undercut + ";\n            }\n";
                any_noncons = any_noncons || nc_bounded;
                os << "        {  // member " << i << "\n";
                // members the exact sphere test never culls (the reference's unbounded members, and
                // the non-conservative ones) skip their exact field where their weak bound clears bd
                const WeakBound wb = cull ? WeakBound{} : weak_bound(o, weak_csg, h->n_csg_ops);
                if (wb.ok) {
                    if (!(o.flags & OF_ROT_IDENTITY)) os << "            const float RO[9] = " << farr(o.rot, 9) << ";\n";
                    exact = "if (!" + weak_cull_expr(o, wb) + ") {\n            " + exact + "            }\n";
                }
                if (o.flags & OF_BOUND) {
                    if (cull) {
                        os << "            if (!" << sphere_test(o.bc, o.br, "bd", false) << ") {\n"
                           << "            const float lower = " << lower_expr(o) << ";\n";
                    } else {
                        // beyond both the slack and bd, the member's value is its sphere distance and
                        // it cannot win: the squared pre-test skips the square root there
                        os << "            if (!" << sphere_test(o.bc, o.br, "fmaxf(bd, " + slack + ")", slack_pos) << ") {\n"
                           << "            const float lower = " << lower_expr(o) << ";\n";
                    }
                    if (cull) os << "            if (!(lower > bd)) {\n";
                    os << "            if (lower > " << slack << ") {\n                if (lower < bd || (lower == bd && "
                       << i << " < bi)) {\n                    bd = lower;\n                    bi = " << i
                       << ";\n                    bm = " << o.mat << "u;\n                    bnc = false;\n"
                       << "                }\n            } else {\n            " << exact << "            }\n";
                    os << (cull ? "            }\n            }\n" : "            }\n");
                } else {
                    os << "            " << exact;
                }
                os << "        }\n";
            };
            // order: members that are always evaluated (they set an early best), the sphere-tested
            // clusters, then the weak-bound members, whose looser bound needs the smallest best
            std::vector<uint32_t> weak;
            for (uint32_t k = 0; k < sg.b; ++k) {
                uint32_t i = unb[sg.a + k];
                bool cull = (obj[i].flags & OF_BOUND) && !(obj[i].flags & OF_NONCONS);
                if (cull) cullable.push_back(i);
                else if (weak_bound(obj[i], weak_csg, h->n_csg_ops).ok) weak.push_back(i);
                else member(i, false);
            }
            std::vector<MemberCluster> clusters;
            cluster_members(obj, cullable, clusters);
            // The clusters and the bounded weak members (whose sphere tests take fmaxf(bd, slack))
            // under one enclosing sphere when there are three or more: where a sample is beyond
            // it, every test inside would cull. Its threshold is fmaxf(bd, slack) when a bounded
            // weak member is inside (no smaller than bd, so it covers the clusters too).
            std::vector<uint32_t> weak_bounded, weak_free;
            for (uint32_t i : weak) ((obj[i].flags & OF_BOUND) ? weak_bounded : weak_free).push_back(i);
            std::vector<std::pair<const float*, float>> spheres;
            for (const MemberCluster& cl : clusters) spheres.push_back({cl.c, cl.r});
            for (uint32_t i : weak_bounded) spheres.push_back({obj[i].bc, obj[i].br});
            float sc[3];
            float sr = 0.0f;
            const bool super = spheres.size() >= 3 && enclosing_sphere(spheres, sc, sr);
            if (super) {
                const std::string thr = weak_bounded.empty() ? std::string("bd") : "fmaxf(bd, " + slack + ")";
                os << "        if (!" << sphere_test(sc, sr, thr, !weak_bounded.empty() && slack_pos)
                   << ") {  // enclosing sphere of " << spheres.size() << " tests, radius " << fbits(sr) << "\n";
            }
            for (const MemberCluster& cl : clusters) {
                if (cl.members.size() > 1)
                    os << "        if (!" << sphere_test(cl.c, cl.r, "bd", false) << ") {  // cluster of " << cl.members.size()
                       << ", radius " << fbits(cl.r) << "\n";
                for (uint32_t i : cl.members) member(i, true);
                if (cl.members.size() > 1) os << "        }  // end of cluster\n";
            }
            for (uint32_t i : weak_bounded) member(i, false);
            if (super) os << "        }  // end of enclosing sphere\n";
            for (uint32_t i : weak_free) member(i, false);
            if (any_noncons)
                os << "        if (bnc) acc = walk_" << s << "(T, p, acc);\n        else acc = Field{bd, bm};\n";
            else
                os << "        (void)bnc;  // no member can undercut its bound\n        acc = Field{bd, bm};\n";
        } else {
            os << "        acc = walk_" << s << "(T, p, acc);\n";
        }
        os << "    }\n";
    }
    os << "    return acc;\n}\n";
    // Scene::normal_dual (lib.rs:820-835) over the scene's objects with their records inlined
    // (only reached when the scene is dual-safe)
    os << "__device__ __forceinline__ V normal_dual(V p) {\n";
    if ((h->flags & SF_DUAL_SAFE) && h->n_objects > 0) {
        os << "    D acc;\n";
        for (uint32_t i = 0; i < h->n_objects; ++i) {
            os << "    {\n        const DevObject o = " << object_rec(obj[i]) << ";\n";
            if (i == 0) os << "        acc = object_dual<true>(o, p);\n";
            else os << "        acc = dual_fold(acc, object_dual<true>(o, p), o.flags, o.k);\n";
            os << "    }\n";
        }
        os << "    return normalize(acc.g);\n}\n";
    } else {
        os << "    return V{0.f, 0.f, 0.f};\n}\n";
    }
    // the field class of the pass bodies: the field above, and the scene's marcher settings as
    // constants (the tape header's values, which the scene's tape keeps while it is specialised)
    auto u = [](uint32_t v) { return std::to_string(v) + "u"; };
    os << "struct Field_ {\n"
          "    static constexpr bool kConstSettings = true;\n"
          "    static __device__ __forceinline__ Field eval(const Tape& T, V p) { return spec::eval(T, p); }\n"
          "    static __device__ __forceinline__ V normal_dual(const Tape&, V p) { return spec::normal_dual(p); }\n"
       << "    static __device__ __forceinline__ uint32_t flags(const TapeHeader&) { return " << u(h->flags) << "; }\n"
       << "    static __device__ __forceinline__ uint32_t max_steps(const TapeHeader&) { return " << u(h->max_steps) << "; }\n"
       << "    static __device__ __forceinline__ uint32_t shadow_steps(const TapeHeader&) { return " << u(h->shadow_steps)
       << "; }\n"
       << "    static __device__ __forceinline__ uint32_t ao_samples(const TapeHeader&) { return " << u(h->ao_samples)
       << "; }\n"
       << "    static __device__ __forceinline__ uint32_t n_lights(const TapeHeader&) { return " << u(h->n_lights) << "; }\n"
       << "    static __device__ __forceinline__ float max_dist(const TapeHeader&) { return " << fbits(h->max_dist) << "; }\n"
       << "    static __device__ __forceinline__ float eps(const TapeHeader&) { return " << fbits(h->eps) << "; }\n"
       << "    static __device__ __forceinline__ float step_scale(const TapeHeader&) { return " << fbits(h->step_scale)
       << "; }\n"
       << "    static __device__ __forceinline__ float lod_footprint(const TapeHeader&) { return " << fbits(h->lod_footprint)
       << "; }\n"
       << "    static __device__ __forceinline__ float subitize(const TapeHeader&) { return " << fbits(h->subitize) << "; }\n"
       << "    static __device__ __forceinline__ float normal_h(const TapeHeader&) { return " << fbits(h->normal_h) << "; }\n"
       << "};\n}  // namespace spec\n}  // namespace mm3e\n";
    const int tm = smem_tape ? 0 : 1;
    // With no explicit register budget both persistent kernels ask for 8 CTAs of 128 (4 of 256)
    // per SM, at most 64 registers: with no function call left in the generated field (the BVH
    // walks are inlined), the gallery's march and shadow fit that without spills (62 / 59), and the
    // extra resident warps hide branch and instruction-fetch latency. (Left to itself, ptxas gave
    // the shadow kernel 64 registers with spills.)
    // The shadow kernel of a small field (at most 16 objects, no CSG program) asks for 10 CTAs of
    // 128 (5 of 256), 48 registers: the gallery's fits without spills and its shadow pass took
    // 0.648 against 0.681 ms per 1080p frame. The fields of larger scenes (the seeded procedural
    // scenes of 8-64 primitives) mostly need fewer registers anyway, and some of them spill at 48.
    const bool small_field = h->n_objects <= 16 && h->n_csg_ops == 0;
    const uint32_t mb = min_blocks ? min_blocks : (block <= 128 ? 8u : 4u);
    const uint32_t mb_shadow = min_blocks ? min_blocks : small_field ? (block <= 128 ? 10u : 5u) : (block <= 128 ? 8u : 4u);
    const std::string march_bounds = std::to_string(block) + ", " + std::to_string(mb);
    const std::string bounds = std::to_string(block) + ", " + std::to_string(mb_shadow);
    os << "extern \"C\" __global__ void __launch_bounds__(" << march_bounds
       << ") mm3e_spec_march(const __grid_constant__ mm3e::WaveArgs a) {\n    mm3e::wave::march_body<" << tm << ", "
       << unroll << ", mm3e::spec::Field_>(a);\n}\n"
       << "extern \"C\" __global__ void __launch_bounds__(" << bounds
       << ") mm3e_spec_shadow(const __grid_constant__ mm3e::WaveArgs a) {\n    mm3e::wave::shadow_body<" << tm << ", "
       << unroll << ", mm3e::spec::Field_>(a);\n}\n"
       << "extern \"C\" __global__ void __launch_bounds__(128) mm3e_spec_ao(const __grid_constant__ mm3e::WaveArgs a) {\n"
          "    mm3e::wave::ao_body<mm3e::spec::Field_>(a);\n}\n";
    return os.str();
}

}  // namespace mm3e
