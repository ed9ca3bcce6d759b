// scene_io.cpp — the `.mm3e` line-oriented text scene format (scene_io.rs): parse into an owned
// scene description + camera, and write one back. Same directives, value order, validation and
// error messages as the reference; numbers are written as the shortest decimal that reads back
// to the same binary32 (Rust's `{}` for f32), so writing what was read gives the same text.
#include <charconv>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"

struct mm3e_parsed_scene {
    mm3e::SceneCopy sc;
    mm3e_camera cam{};
};

namespace {

using mm3e::SceneCopy;

struct P3 {
    float x, y, z;
};
P3 sub3(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
float dot3(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
P3 cross3(P3 a, P3 o) { return {a.y * o.z - a.z * o.y, a.z * o.x - a.x * o.z, a.x * o.y - a.y * o.x}; }
P3 norm3(P3 a) {  // vec.rs:37-44
    float len = std::sqrt(dot3(a, a));
    return len > 1e-12f ? P3{a.x * (1.0f / len), a.y * (1.0f / len), a.z * (1.0f / len)} : P3{0, 0, 0};
}
bool zero3(P3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }

// Scene::new defaults (mm3e-orchestrator/src/lib.rs:595-620; post.rs:25-29; march.rs:81-96).
void scene_defaults(SceneCopy& sc, uint32_t w, uint32_t h) {
    mm3e_scene_desc& d = sc.d;
    d = mm3e_scene_desc{};
    d.width = w;
    d.height = h;
    P3 sun = norm3({0.6f, 0.7f, 0.4f});
    d.sun_dir[0] = sun.x;
    d.sun_dir[1] = sun.y;
    d.sun_dir[2] = sun.z;
    for (int i = 0; i < 3; ++i) {
        d.ambient[i] = 0.02f;
        d.sky_ambient[i] = 0.4f;
    }
    d.fog[0] = 0.62f;
    d.fog[1] = 0.72f;
    d.fog[2] = 0.86f;
    d.fog_density = 0.012f;
    d.aa = 2;
    d.bounces = 1;
    d.shadows = 1;
    d.ao = 1;
    d.marcher.max_steps = 160;
    d.marcher.max_dist = 120.0f;
    d.marcher.eps = 0.0006f;
    d.marcher.step_scale = 1.0f;
    d.marcher.shadow_steps = 64;
    d.marcher.ao_samples = 5;
    d.marcher.lod_footprint = 0.0f;
    d.marcher.subitize = 0.0f;
    d.marcher.secant = 0;
    d.marcher.normal_h = 0.0009f;
    d.post.exposure = 1.0f;
    d.post.bloom = 1;
    d.post.bloom_threshold = 1.0f;
    d.post.bloom_intensity = 0.06f;
    d.post.bloom_radius = 12;
    d.mode = MM3E_MODE_BEAUTY;
    sc.objects.clear();
    sc.materials.clear();
    sc.lights.clear();
}

mm3e_material default_material() {  // Material::default (color.rs)
    mm3e_material m{};
    m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.8f;
    m.metallic = 0.0f;
    m.specular = 0.5f;
    m.roughness = 0.35f;
    m.reflectivity = 0.0f;
    m.checker = 0;
    return m;
}

// Camera::look_at (camera.rs:50-55)
mm3e_camera look_at(P3 eye, P3 target, P3 up_hint, float fov_y) {
    P3 fwd = norm3(sub3(target, eye));
    P3 right = norm3(cross3(fwd, up_hint));
    P3 up = cross3(right, fwd);
    mm3e_camera c{};
    std::memcpy(c.eye, &eye, 12);
    std::memcpy(c.forward, &fwd, 12);
    std::memcpy(c.right, &right, 12);
    std::memcpy(c.up, &up, 12);
    c.fov_scale = std::tan(fov_y * 0.5f);
    return c;
}

struct Cur {
    const char* p;
    const char* end;
    size_t line;
    std::string err;
    bool next(const char* what, std::string& out) {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\f' || *p == '\v')) ++p;
        if (p >= end) {
            err = "line " + std::to_string(line) + ": expected " + what;
            return false;
        }
        const char* s = p;
        while (p < end && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\f' || *p == '\v')) ++p;
        out.assign(s, p);
        return true;
    }
    bool has_more() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\f' || *p == '\v')) ++p;
        return p < end;
    }
    // str::parse::<f32> then the finite check
    bool f(const char* what, float& v) {
        std::string t;
        if (!next(what, t)) return false;
        const char* b = t.data();
        const char* e = t.data() + t.size();
        bool neg = false;
        if (b < e && (*b == '+' || *b == '-')) {
            neg = *b == '-';
            ++b;
        }
        float x = 0.0f;
        auto r = std::from_chars(b, e, x, std::chars_format::general);
        bool ok = r.ec == std::errc() && r.ptr == e && b < e;
        if (!ok) {  // inf / infinity / nan spellings parse too, then fail the finite check
            std::string low;
            for (const char* q = b; q < e; ++q) low += (char)std::tolower((unsigned char)*q);
            if (low == "inf" || low == "infinity" || low == "nan") {
                err = "line " + std::to_string(line) + ": non-finite number '" + t + "' for " + what;
                return false;
            }
            err = "line " + std::to_string(line) + ": bad number '" + t + "' for " + what;
            return false;
        }
        v = neg ? -x : x;
        if (!std::isfinite(v)) {
            err = "line " + std::to_string(line) + ": non-finite number '" + t + "' for " + what;
            return false;
        }
        return true;
    }
    bool u(const char* what, uint32_t& v) {
        std::string t;
        if (!next(what, t)) return false;
        const char* b = t.data();
        const char* e = t.data() + t.size();
        if (b < e && *b == '+') ++b;
        auto r = std::from_chars(b, e, v);
        if (r.ec != std::errc() || r.ptr != e || b == e) {
            err = "line " + std::to_string(line) + ": bad integer '" + t + "' for " + what;
            return false;
        }
        return true;
    }
    bool bo(const char* what, uint32_t& v) {
        uint32_t x;
        if (!u(what, x)) return false;
        v = x != 0 ? 1u : 0u;
        return true;
    }
    bool v3(const char* what, float* out) { return f(what, out[0]) && f(what, out[1]) && f(what, out[2]); }
};

bool positive3(const float* v) { return v[0] > 0.0f && v[1] > 0.0f && v[2] > 0.0f; }

// validate_prim (scene_io.rs:283-307); params layout as mm3e_object.params.
std::string validate_prim(size_t line, const mm3e_object& o) {
    const float* q = o.params;
    auto bad = [&](const char* msg) { return "line " + std::to_string(line) + ": " + msg; };
    switch (o.prim) {
        case MM3E_PRIM_SPHERE: return q[0] <= 0.0f ? bad("sphere radius must be positive") : "";
        case MM3E_PRIM_BOX: return !positive3(q) ? bad("box half extents must be positive") : "";
        case MM3E_PRIM_ROUND_BOX:
            return (!positive3(q) || q[3] < 0.0f) ? bad("roundbox half extents must be positive and radius non-negative")
                                                  : "";
        case MM3E_PRIM_TORUS: return (q[0] <= 0.0f || q[1] <= 0.0f) ? bad("torus radii must be positive") : "";
        case MM3E_PRIM_CYLINDER:
            return (q[0] <= 0.0f || q[1] <= 0.0f) ? bad("cylinder height and radius must be positive") : "";
        case MM3E_PRIM_CAPSULE: {
            P3 d = sub3({q[3], q[4], q[5]}, {q[0], q[1], q[2]});
            return (q[6] <= 0.0f || std::sqrt(dot3(d, d)) <= 1e-6f)
                       ? bad("capsule radius must be positive and endpoints must differ")
                       : "";
        }
        case MM3E_PRIM_CONE:
            return (q[0] < 0.0f || q[1] < 0.0f || q[2] <= 0.0f || (q[0] == 0.0f && q[1] == 0.0f))
                       ? bad("cone height must be positive and at least one radius must be positive")
                       : "";
        case MM3E_PRIM_ELLIPSOID: return !positive3(q) ? bad("ellipsoid radii must be positive") : "";
        case MM3E_PRIM_OCTAHEDRON: return q[0] <= 0.0f ? bad("octahedron size must be positive") : "";
        case MM3E_PRIM_HEX_PRISM:
            return (q[0] <= 0.0f || q[1] <= 0.0f) ? bad("hex prism radius and height must be positive") : "";
        case MM3E_PRIM_PLANE: return zero3(norm3({q[0], q[1], q[2]})) ? bad("plane normal must be non-zero") : "";
        default: return "";
    }
}

struct PrimName {
    const char* name;
    uint32_t prim;
    int nparams;
};
const PrimName kPrims[] = {{"sphere", MM3E_PRIM_SPHERE, 1},     {"box", MM3E_PRIM_BOX, 3},
                           {"roundbox", MM3E_PRIM_ROUND_BOX, 4}, {"torus", MM3E_PRIM_TORUS, 2},
                           {"cylinder", MM3E_PRIM_CYLINDER, 2},  {"capsule", MM3E_PRIM_CAPSULE, 7},
                           {"cone", MM3E_PRIM_CONE, 3},          {"ellipsoid", MM3E_PRIM_ELLIPSOID, 3},
                           {"octahedron", MM3E_PRIM_OCTAHEDRON, 1}, {"hexprism", MM3E_PRIM_HEX_PRISM, 2},
                           {"plane", MM3E_PRIM_PLANE, 4}};

// parse_object (scene_io.rs:309-355)
bool parse_object(Cur& c, mm3e_object& o) {
    std::string name;
    if (!c.next("primitive", name)) return false;
    const PrimName* pn = nullptr;
    for (const PrimName& k : kPrims)
        if (name == k.name) pn = &k;
    if (!pn) {
        c.err = "line " + std::to_string(c.line) + ": unknown primitive '" + name + "'";
        return false;
    }
    o = mm3e_object{};
    o.prim = pn->prim;
    static const char* pnames[][7] = {{"r"}, {"half", "half", "half"}, {"half", "half", "half", "radius"},
                                      {"major", "minor"}, {"h", "r"}, {"a", "a", "a", "b", "b", "b", "r"},
                                      {"r1", "r2", "h"}, {"r", "r", "r"}, {"s"}, {"r", "h"}, {"n", "n", "n", "h"}};
    for (int i = 0; i < pn->nparams; ++i)
        if (!c.f(pnames[pn - kPrims][i], o.params[i])) return false;
    std::string verr = validate_prim(c.line, o);
    if (!verr.empty()) {
        c.err = verr;
        return false;
    }
    float pos[3] = {0, 0, 0};
    float basis[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    float scale = 1.0f;
    o.combine = MM3E_COMBINE_UNION;
    while (c.has_more()) {
        std::string kw;
        c.next("modifier or end", kw);
        if (kw == "pos") {
            if (!c.v3("pos", pos)) return false;
        } else if (kw == "basis") {
            if (!c.v3("col0", basis) || !c.v3("col1", basis + 3) || !c.v3("col2", basis + 6)) return false;
        } else if (kw == "scale") {
            if (!c.f("scale", scale)) return false;
            if (scale <= 0.0f) {
                c.err = "line " + std::to_string(c.line) + ": object scale must be positive";
                return false;
            }
        } else if (kw == "mat") {
            if (!c.u("mat", o.mat)) return false;
        } else if (kw == "combine") {
            std::string k;
            if (!c.next("combine kind", k)) return false;
            if (k == "union") o.combine = MM3E_COMBINE_UNION;
            else if (k == "smooth") {
                o.combine = MM3E_COMBINE_SMOOTH;
                if (!c.f("k", o.smooth_k)) return false;
            } else if (k == "subtract") o.combine = MM3E_COMBINE_SUBTRACT;
            else {
                c.err = "line " + std::to_string(c.line) + ": unknown combine '" + k + "'";
                return false;
            }
        } else if (kw == "round") {
            if (!c.f("round", o.round)) return false;
        } else if (kw == "onion") {
            if (!c.f("onion", o.onion)) return false;
        } else if (kw == "twist") {
            if (!c.f("twist", o.twist)) return false;
        } else if (kw == "bend") {
            if (!c.f("bend", o.bend)) return false;
        } else if (kw == "mirror") {
            uint32_t mx, my, mz;
            if (!c.bo("mx", mx) || !c.bo("my", my) || !c.bo("mz", mz)) return false;
            o.mirror = mx | (my << 1) | (mz << 2);
        } else if (kw == "repeat") {
            if (!c.v3("repeat", o.repeat)) return false;
        } else if (kw == "elongate") {
            if (!c.v3("elongate", o.elongate)) return false;
        } else {
            c.err = "line " + std::to_string(c.line) + ": unknown object field '" + kw + "'";
            return false;
        }
    }
    std::memcpy(o.rot, basis, sizeof basis);
    std::memcpy(o.pos, pos, sizeof pos);
    o.scale = scale;
    return true;
}

std::string fmt(float v) {  // Rust `{}` for f32: shortest round-trip decimal, no exponent
    char b[64];
    auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::fixed);
    std::string s(b, r.ptr);
    if (s == "-0") s = "-0";
    return s;
}
std::string fmt3(const float* v) { return fmt(v[0]) + " " + fmt(v[1]) + " " + fmt(v[2]); }

const char* mode_name(uint32_t m) {
    switch (m) {
        case MM3E_MODE_NORMAL: return "normal";
        case MM3E_MODE_DEPTH: return "depth";
        case MM3E_MODE_AO: return "ao";
        case MM3E_MODE_STEPS: return "steps";
        case MM3E_MODE_ALBEDO: return "albedo";
        default: return "beauty";
    }
}

void put_err(const std::string& e, char* err, size_t err_len) {
    if (err && err_len) {
        std::strncpy(err, e.c_str(), err_len - 1);
        err[err_len - 1] = 0;
    }
}

// ---- .sdfv (volume.rs:115-187, 230-248) ----------------------------------------------------
constexpr size_t SDFV_HEADER = 8 + 3 * 4 + 3 * 4 + 3 * 4;
const char SDFV_MAGIC[9] = "MM3ESDF1";

uint32_t le_u32(const uint8_t* b) {
    return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}
void put_le_u32(uint8_t* b, uint32_t v) {
    b[0] = (uint8_t)v;
    b[1] = (uint8_t)(v >> 8);
    b[2] = (uint8_t)(v >> 16);
    b[3] = (uint8_t)(v >> 24);
}
float f32_of(uint32_t bits) {
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}
uint32_t bits_of(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// SdfVolume::validate_layout (volume.rs:62-87): dims, min and cell rules (the data length is
// implied by the dims in this interface).
std::string layout_error(uint64_t nx, uint64_t ny, uint64_t nz, const float* mn, const float* cell) {
    if (nx < 2 || ny < 2 || nz < 2) return "SdfVolume dims must all be >= 2";
    if (!(std::isfinite(mn[0]) && std::isfinite(mn[1]) && std::isfinite(mn[2]))) return "SdfVolume min must be finite";
    if (!(std::isfinite(cell[0]) && std::isfinite(cell[1]) && std::isfinite(cell[2])) ||
        !(cell[0] > 0.0f && cell[1] > 0.0f && cell[2] > 0.0f))
        return "SdfVolume cell sizes must be positive and finite";
    return "";
}

bool mul_overflows(uint64_t a, uint64_t b, uint64_t& r) {
    if (a != 0 && b > UINT64_MAX / a) return true;
    r = a * b;
    return false;
}

}  // namespace

extern "C" {

// scene_io::parse (scene_io.rs:196-281)
int mm3e_scene_parse_mm3e(const char* text, mm3e_parsed_scene** out, char* err, size_t err_len) {
    if (!text || !out) return MM3E_ERR_INVALID;
    *out = nullptr;
    std::unique_ptr<mm3e_parsed_scene> ps(new mm3e_parsed_scene());
    SceneCopy& sc = ps->sc;
    scene_defaults(sc, 640, 360);
    ps->cam = look_at({0.0f, 1.0f, 6.0f}, {0, 0, 0}, {0.0f, 1.0f, 0.0f}, 1.0f);
    mm3e_scene_desc& d = sc.d;
    const char* p = text;
    const char* end = text + std::strlen(text);
    size_t lineno = 0;
    auto failp = [&](const std::string& e) {
        put_err(e, err, err_len);
        return MM3E_ERR_INVALID;
    };
    while (p <= end) {
        const char* eol = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
        if (!eol) eol = end;
        ++lineno;
        const char* hash = static_cast<const char*>(std::memchr(p, '#', (size_t)(eol - p)));
        Cur c{p, hash ? hash : eol, lineno, ""};
        p = eol + 1;
        if (!c.has_more()) {
            if (eol == end) break;
            continue;
        }
        std::string dir;
        c.next("directive", dir);
        std::string L = "line " + std::to_string(lineno) + ": ";
        bool ok = true;
        if (dir == "size") {
            ok = c.u("width", d.width) && c.u("height", d.height);
            if (ok && (d.width == 0 || d.height == 0 || d.width > 16384 || d.height > 16384))
                return failp(L + "size " + std::to_string(d.width) + "x" + std::to_string(d.height) +
                             " out of range 1..=16384");
        } else if (dir == "aa") {
            ok = c.u("aa", d.aa);
        } else if (dir == "bounces") {
            ok = c.u("bounces", d.bounces);
        } else if (dir == "shadows") {
            ok = c.bo("shadows", d.shadows);
        } else if (dir == "ao") {
            ok = c.bo("ao", d.ao);
        } else if (dir == "sun") {
            float v[3];
            ok = c.v3("sun", v);
            if (ok) {
                P3 n = norm3({v[0], v[1], v[2]});
                if (zero3(n)) return failp(L + "sun direction must be non-zero");
                d.sun_dir[0] = n.x;
                d.sun_dir[1] = n.y;
                d.sun_dir[2] = n.z;
            }
        } else if (dir == "ambient") {
            ok = c.v3("ambient", d.ambient);
        } else if (dir == "sky_ambient") {
            ok = c.v3("sky_ambient", d.sky_ambient);
        } else if (dir == "fog") {
            ok = c.v3("fog", d.fog) && c.f("fog density", d.fog_density);
        } else if (dir == "marcher") {
            ok = c.u("max_steps", d.marcher.max_steps) && c.f("max_dist", d.marcher.max_dist) &&
                 c.f("eps", d.marcher.eps) && c.f("step_scale", d.marcher.step_scale);
            if (ok && (d.marcher.max_steps == 0 || d.marcher.max_steps > 100000))
                return failp(L + "marcher max_steps out of range 1..=100000");
            if (ok && !(d.marcher.max_dist > 0.0f && d.marcher.eps > 0.0f && d.marcher.step_scale > 0.0f))
                return failp(L + "marcher max_dist/eps/step_scale must be positive");
        } else if (dir == "post") {
            ok = c.f("exposure", d.post.exposure) && c.bo("bloom", d.post.bloom) &&
                 c.f("bloom_threshold", d.post.bloom_threshold) && c.f("bloom_intensity", d.post.bloom_intensity) &&
                 c.u("bloom_radius", d.post.bloom_radius);
        } else if (dir == "mode") {
            std::string m;
            ok = c.next("mode", m);
            if (ok) {
                if (m == "beauty") d.mode = MM3E_MODE_BEAUTY;
                else if (m == "normal") d.mode = MM3E_MODE_NORMAL;
                else if (m == "depth") d.mode = MM3E_MODE_DEPTH;
                else if (m == "ao") d.mode = MM3E_MODE_AO;
                else if (m == "steps") d.mode = MM3E_MODE_STEPS;
                else if (m == "albedo") d.mode = MM3E_MODE_ALBEDO;
                else return failp(L + "unknown render mode '" + m + "'");
            }
        } else if (dir == "cam") {
            float eye[3], target[3], up[3], fov;
            ok = c.v3("eye", eye) && c.v3("target", target) && c.v3("up", up) && c.f("fov", fov);
            if (ok) {
                P3 e{eye[0], eye[1], eye[2]}, t{target[0], target[1], target[2]}, u{up[0], up[1], up[2]};
                P3 fwd = norm3(sub3(t, e));
                if (zero3(fwd)) return failp(L + "cam eye and target must not coincide");
                if (zero3(norm3(cross3(fwd, u)))) return failp(L + "cam up must not be parallel to the view direction");
                if (!(fov > 0.0f) || fov >= 180.0f) return failp(L + "cam fov must be in (0, 180) degrees");
                const float rads_per_deg = 3.14159265358979323846f / 180.0f;  // f32::to_radians
                ps->cam = look_at(e, t, u, fov * rads_per_deg);
            }
        } else if (dir == "mat") {
            mm3e_material m{};
            ok = c.v3("albedo", m.albedo) && c.f("metallic", m.metallic) && c.f("roughness", m.roughness) &&
                 c.f("reflectivity", m.reflectivity) && c.f("specular", m.specular) && c.v3("emissive", m.emissive) &&
                 c.bo("checker", m.checker);
            if (ok) sc.materials.push_back(m);
        } else if (dir == "light") {
            std::string kind;
            mm3e_light l{};
            ok = c.next("light kind", kind) && c.v3("light vec", l.vec) && c.v3("light color", l.color) &&
                 c.f("light radius", l.radius);
            if (ok) {
                if (kind == "dir") l.directional = 1;
                else if (kind == "point") l.directional = 0;
                else return failp(L + "unknown light kind '" + kind + "'");
                sc.lights.push_back(l);
            }
        } else if (dir == "obj") {
            mm3e_object o{};
            ok = parse_object(c, o);
            if (ok) sc.objects.push_back(o);
        } else {
            return failp(L + "unknown directive '" + dir + "'");
        }
        if (!ok) return failp(c.err);
        if (eol == end) break;
    }
    if (sc.materials.empty()) sc.materials.push_back(default_material());
    for (size_t i = 0; i < sc.objects.size(); ++i)
        if (sc.objects[i].mat >= sc.materials.size())
            return failp("object " + std::to_string(i + 1) + ": material index " + std::to_string(sc.objects[i].mat) +
                         " out of range (have " + std::to_string(sc.materials.size()) + ")");
    d.n_objects = (uint32_t)sc.objects.size();
    d.n_materials = (uint32_t)sc.materials.size();
    d.n_lights = (uint32_t)sc.lights.size();
    sc.fix();
    *out = ps.release();
    return MM3E_OK;
}

const mm3e_scene_desc* mm3e_parsed_scene_desc(const mm3e_parsed_scene* ps) { return ps ? &ps->sc.d : nullptr; }

int mm3e_parsed_scene_camera(const mm3e_parsed_scene* ps, mm3e_camera* out) {
    if (!ps || !out) return MM3E_ERR_INVALID;
    *out = ps->cam;
    return MM3E_OK;
}

void mm3e_parsed_scene_free(mm3e_parsed_scene* ps) { delete ps; }

// scene_io::try_serialize (scene_io.rs:38-95)
int mm3e_scene_write_mm3e(const mm3e_scene_desc* d, const mm3e_camera* cam, char* out, size_t cap, size_t* len,
                          char* err, size_t err_len) {
    if (!d || !cam) return MM3E_ERR_INVALID;
    for (uint32_t i = 0; i < d->n_objects; ++i) {
        if (d->objects[i].prim == MM3E_PRIM_SURFACE) {
            put_err("triangle surfaces are not representable in the legacy .mm3e text format; use the durable editor "
                    "format",
                    err, err_len);
            return MM3E_ERR_UNSUPPORTED;
        }
        if (d->objects[i].prim == MM3E_PRIM_CSG) {
            put_err("object-local CSG is not representable in the legacy .mm3e text format", err, err_len);
            return MM3E_ERR_UNSUPPORTED;
        }
    }
    std::string s = "# MM3E scene\n";
    s += "size " + std::to_string(d->width) + " " + std::to_string(d->height) + "\n";
    s += "aa " + std::to_string(d->aa) + "\n";
    s += "bounces " + std::to_string(d->bounces) + "\n";
    s += "shadows " + std::to_string(d->shadows ? 1 : 0) + "\n";
    s += "ao " + std::to_string(d->ao ? 1 : 0) + "\n";
    s += "sun " + fmt3(d->sun_dir) + "\n";
    s += "ambient " + fmt3(d->ambient) + "\n";
    s += "sky_ambient " + fmt3(d->sky_ambient) + "\n";
    s += "fog " + fmt3(d->fog) + " " + fmt(d->fog_density) + "\n";
    s += "marcher " + std::to_string(d->marcher.max_steps) + " " + fmt(d->marcher.max_dist) + " " +
         fmt(d->marcher.eps) + " " + fmt(d->marcher.step_scale) + "\n";
    s += "post " + fmt(d->post.exposure) + " " + std::to_string(d->post.bloom ? 1 : 0) + " " +
         fmt(d->post.bloom_threshold) + " " + fmt(d->post.bloom_intensity) + " " + std::to_string(d->post.bloom_radius) +
         "\n";
    s += std::string("mode ") + mode_name(d->mode) + "\n";
    // camera: eye, target = eye + forward, up, vertical FOV in degrees
    float target[3] = {cam->eye[0] + cam->forward[0], cam->eye[1] + cam->forward[1], cam->eye[2] + cam->forward[2]};
    const float pis_in_180 = 57.2957795130823208767981548141051703f;  // f32::to_degrees
    float fov_deg = (std::atan(cam->fov_scale) * 2.0f) * pis_in_180;
    s += "cam " + fmt3(cam->eye) + " " + fmt3(target) + " " + fmt3(cam->up) + " " + fmt(fov_deg) + "\n";
    for (uint32_t i = 0; i < d->n_materials; ++i) {
        const mm3e_material& m = d->materials[i];
        s += "mat " + fmt3(m.albedo) + " " + fmt(m.metallic) + " " + fmt(m.roughness) + " " + fmt(m.reflectivity) + " " +
             fmt(m.specular) + " " + fmt3(m.emissive) + " " + std::to_string(m.checker ? 1 : 0) + "\n";
    }
    for (uint32_t i = 0; i < d->n_lights; ++i) {
        const mm3e_light& l = d->lights[i];
        s += std::string("light ") + (l.directional ? "dir" : "point") + " " + fmt3(l.vec) + " " + fmt3(l.color) + " " +
             fmt(l.radius) + "\n";
    }
    for (uint32_t i = 0; i < d->n_objects; ++i) {
        const mm3e_object& o = d->objects[i];
        if (o.prim == MM3E_PRIM_VOLUME) {
            s += "# volume object omitted (baked SDF volume id " + std::to_string(o.id) + " is not text-serializable)\n";
            continue;
        }
        const PrimName* pn = nullptr;
        for (const PrimName& k : kPrims)
            if (k.prim == o.prim) pn = &k;
        if (!pn) continue;
        s += std::string("obj ") + pn->name;
        for (int k = 0; k < pn->nparams; ++k) s += " " + fmt(o.params[k]);
        s += " pos " + fmt3(o.pos) + " basis " + fmt3(o.rot) + " " + fmt3(o.rot + 3) + " " + fmt3(o.rot + 6) + " scale " +
             fmt(o.scale) + " mat " + std::to_string(o.mat);
        if (o.combine == MM3E_COMBINE_SMOOTH) s += " combine smooth " + fmt(o.smooth_k);
        else if (o.combine == MM3E_COMBINE_SUBTRACT) s += " combine subtract";
        else s += " combine union";
        if (o.round != 0.0f) s += " round " + fmt(o.round);
        if (o.onion != 0.0f) s += " onion " + fmt(o.onion);
        if (o.twist != 0.0f) s += " twist " + fmt(o.twist);
        if (o.bend != 0.0f) s += " bend " + fmt(o.bend);
        if (o.mirror)
            s += " mirror " + std::to_string(o.mirror & 1u) + " " + std::to_string((o.mirror >> 1) & 1u) + " " +
                 std::to_string((o.mirror >> 2) & 1u);
        if (o.repeat[0] != 0.0f || o.repeat[1] != 0.0f || o.repeat[2] != 0.0f) s += " repeat " + fmt3(o.repeat);
        if (o.elongate[0] != 0.0f || o.elongate[1] != 0.0f || o.elongate[2] != 0.0f)
            s += " elongate " + fmt3(o.elongate);
        s += "\n";
    }
    if (len) *len = s.size();
    if (out && cap) {
        size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
        std::memcpy(out, s.data(), n);
        out[n] = 0;
    }
    return MM3E_OK;
}

// SdfVolume::from_sdfv_bytes (volume.rs:140-176)
int mm3e_volume_parse_sdfv(const uint8_t* bytes, size_t n, mm3e_volume* out, float* data, size_t data_cap,
                           size_t* n_samples, char* err, size_t err_len) {
    if ((!bytes && n) || !out) return MM3E_ERR_INVALID;
    auto failp = [&](const std::string& e) {
        put_err(e, err, err_len);
        return MM3E_ERR_INVALID;
    };
    if (n < SDFV_HEADER) return failp("sdfv buffer is shorter than the header");
    if (std::memcmp(bytes, SDFV_MAGIC, 8) != 0) return failp("sdfv magic/version mismatch");
    uint32_t dims[3] = {le_u32(bytes + 8), le_u32(bytes + 12), le_u32(bytes + 16)};
    static const char* names[6] = {"min.x", "min.y", "min.z", "cell.x", "cell.y", "cell.z"};
    float hv[6];
    for (int i = 0; i < 6; ++i) {
        hv[i] = f32_of(le_u32(bytes + 20 + 4 * i));
        if (!std::isfinite(hv[i])) return failp(std::string("sdfv non-finite f32 while reading ") + names[i]);
    }
    uint64_t nxy, samples, payload;
    if (mul_overflows(dims[0], dims[1], nxy) || mul_overflows(nxy, dims[2], samples))
        return failp("sdfv dimensions overflow");
    if (mul_overflows(samples, 4, payload) || payload > UINT64_MAX - SDFV_HEADER)
        return failp("sdfv payload length overflows");
    uint64_t expected = SDFV_HEADER + payload;
    if ((uint64_t)n != expected)
        return failp("sdfv byte length " + std::to_string(n) + " does not match expected " + std::to_string(expected));
    if (n_samples) *n_samples = (size_t)samples;
    for (uint64_t i = 0; i < samples; ++i) {
        uint32_t b = le_u32(bytes + SDFV_HEADER + 4 * i);
        if (!std::isfinite(f32_of(b))) return failp("sdfv non-finite f32 while reading sample " + std::to_string(i));
    }
    // SdfVolume::new: dims and cell rules (the samples are finite by now)
    std::string e = layout_error(dims[0], dims[1], dims[2], hv, hv + 3);
    if (!e.empty()) return failp(e);
    out->nx = dims[0];
    out->ny = dims[1];
    out->nz = dims[2];
    for (int i = 0; i < 3; ++i) {
        out->min[i] = hv[i];
        out->cell[i] = hv[3 + i];
    }
    out->data = data;
    if (!data) return MM3E_OK;
    if (data_cap < samples) return failp("sdfv sample buffer holds " + std::to_string(data_cap) + " of " +
                                         std::to_string(samples) + " samples");
    for (uint64_t i = 0; i < samples; ++i) data[i] = f32_of(le_u32(bytes + SDFV_HEADER + 4 * i));
    return MM3E_OK;
}

// SdfVolume::to_sdfv_bytes (volume.rs:119-137)
int mm3e_volume_write_sdfv(const mm3e_volume* v, uint8_t* out, size_t cap, size_t* len, char* err, size_t err_len) {
    if (!v) return MM3E_ERR_INVALID;
    uint64_t nxy, samples;
    if (mul_overflows(v->nx, v->ny, nxy) || mul_overflows(nxy, v->nz, samples)) {
        put_err("SdfVolume dimensions overflow", err, err_len);
        return MM3E_ERR_INVALID;
    }
    if (!v->data && samples) {
        put_err("SdfVolume data is missing", err, err_len);
        return MM3E_ERR_INVALID;
    }
    std::string e = layout_error(v->nx, v->ny, v->nz, v->min, v->cell);
    for (uint64_t i = 0; e.empty() && i < samples; ++i)  // SdfVolume::validate (volume.rs:33-39)
        if (!std::isfinite(v->data[i])) e = "SdfVolume sample " + std::to_string(i) + " is non-finite";
    if (!e.empty()) {
        put_err(e, err, err_len);
        return MM3E_ERR_INVALID;
    }
    uint64_t total = SDFV_HEADER + 4 * samples;
    if (len) *len = (size_t)total;
    if (!out) return MM3E_OK;
    if (cap < total) {
        put_err("sdfv output buffer holds " + std::to_string(cap) + " of " + std::to_string(total) + " bytes", err,
                err_len);
        return MM3E_ERR_INVALID;
    }
    std::memcpy(out, SDFV_MAGIC, 8);
    put_le_u32(out + 8, v->nx);
    put_le_u32(out + 12, v->ny);
    put_le_u32(out + 16, v->nz);
    for (int i = 0; i < 3; ++i) {
        put_le_u32(out + 20 + 4 * i, bits_of(v->min[i]));
        put_le_u32(out + 32 + 4 * i, bits_of(v->cell[i]));
    }
    for (uint64_t i = 0; i < samples; ++i) put_le_u32(out + SDFV_HEADER + 4 * i, bits_of(v->data[i]));
    return MM3E_OK;
}

}  // extern "C"
