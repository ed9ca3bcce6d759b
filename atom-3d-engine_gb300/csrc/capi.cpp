// capi.cpp — the C ABI (include/mm3e_cuda.h): contexts, compiled scenes and frame rendering.
//
// A context owns one CUDA stream on one device. A compiled scene owns its device tape, the
// uploaded payloads (SDF volume samples, GI probe cubes), its pass buffers (ray queues, hit
// records, HDR and bloom arrays), an output framebuffer and a pinned staging buffer for host
// copies, so a render call allocates nothing. Host-side arithmetic that mirrors Rust
// constructors is binary32 without contraction (this file is compiled with -ffp-contract=off).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "batch.h"
#include "capi_internal.h"
#include "noalloc.h"
#include "spec.h"

using namespace mm3e;

mm3e_ctx::~mm3e_ctx() = default;

namespace mm3e {

void SceneCopy::assign(const mm3e_scene_desc& s) {
    d = s;
    objects.assign(s.objects, s.objects + s.n_objects);
    materials.assign(s.materials, s.materials + s.n_materials);
    lights.assign(s.lights, s.lights + s.n_lights);
    volumes.assign(s.volumes, s.volumes + s.n_volumes);
    volume_data.resize(s.n_volumes);
    for (uint32_t i = 0; i < s.n_volumes; ++i) {
        size_t n = (size_t)s.volumes[i].nx * s.volumes[i].ny * s.volumes[i].nz;
        volume_data[i].assign(s.volumes[i].data, s.volumes[i].data + n);
    }
    csg_nodes.assign(s.csg_nodes, s.csg_nodes + s.n_csg_nodes);
    csg_roots.assign(s.csg_roots, s.csg_roots + s.n_csgs);
    has_gi = s.gi != nullptr;
    if (has_gi) {
        gi = *s.gi;
        size_t n = (size_t)gi.nx * gi.ny * gi.nz * 18;
        gi_cubes.assign(s.gi->cubes, s.gi->cubes + n);
    }
    fix();
}

void SceneCopy::fix() {
    d.objects = objects.data();
    d.materials = materials.data();
    d.lights = lights.data();
    for (size_t i = 0; i < volumes.size(); ++i) volumes[i].data = volume_data[i].data();
    d.volumes = volumes.data();
    d.csg_nodes = csg_nodes.data();
    d.csg_roots = csg_roots.data();
    if (has_gi) {
        gi.cubes = gi_cubes.data();
        d.gi = &gi;
    } else {
        d.gi = nullptr;
    }
}

int fail(mm3e_ctx* c, int code, const std::string& msg) {
    static std::mutex mu;  // a server's worker and its clients may report errors concurrently
    if (c) {
        std::lock_guard<std::mutex> lk(mu);
        c->err = msg;
    }
    return code;
}

int cuda_fail(mm3e_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? MM3E_ERR_NO_MEMORY : MM3E_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

void fill_camera(CameraArgs& a, const mm3e_camera& c) {
    std::memcpy(a.eye, c.eye, 12);
    std::memcpy(a.fwd, c.forward, 12);
    std::memcpy(a.right, c.right, 12);
    std::memcpy(a.up, c.up, 12);
    a.fov_scale = c.fov_scale;
}

FrameJob scene_job(const mm3e_scene* s, const unsigned char* tape, const mm3e_camera& cam, uint32_t w, uint32_t h,
                   uint32_t wlog) {
    FrameJob j{};
    j.tape = tape ? tape : s->d_tape;
    j.bloom_w = s->d_kernel;
    fill_camera(j.cam, cam);
    j.width = w ? w : s->low.width;
    j.height = h ? h : s->low.height;
    j.aa = s->low.aa;
    j.spp = j.aa * j.aa;
    j.tiles_x = tiles_x_of(j.width, wlog);
    j.n_slots = (uint32_t)slots_of(j.width, j.height, wlog);
    j.n_samples = j.n_slots * j.spp;
    j.n_pixels = j.width * j.height;
    j.n_lights = s->n_lights();
    const mm3e_post& post = s->src.d.post;
    j.bloom_radius = s->bloom_radius;
    j.flags = (post.bloom && post.bloom_intensity > 0.0f) ? JF_BLOOM : 0u;
    j.threshold = post.bloom_threshold;
    j.intensity = post.bloom_intensity;
    j.exposure = post.exposure;
    j.format = MM3E_FB_RGBA8;
    return j;
}

PassPlan plain_plan(const mm3e_scene* s, const mm3e_camera& cam, uint32_t w, uint32_t h, uint32_t format, void* dout,
                    uint32_t wlog) {
    const TapeHeader* hd = reinterpret_cast<const TapeHeader*>(s->low.blob.data());
    PassPlan p;
    p.job0 = scene_job(s, nullptr, cam, w, h, wlog);
    p.job0.format = format;
    p.job0.out = dout;
    p.tape_bytes = (uint32_t)s->low.blob.size();
    p.n_samples = p.job0.n_samples;
    p.n_slots = p.job0.n_slots;
    p.n_pixels = p.job0.n_pixels;
    p.levels = s->low.bounces + 1;
    p.lights_max = hd->n_lights;
    p.ao = (hd->flags & SF_AO) && hd->ao_samples > 0;
    p.shadows = (hd->flags & SF_SHADOWS) && hd->shadow_steps > 0 && hd->n_lights > 0;
    p.bloom = (p.job0.flags & JF_BLOOM) != 0;
    p.wait_limit = s->ctx->wait_limit;
    p.wait_probe = s->ctx->wait_probe;
    return p;
}

}  // namespace mm3e

uint32_t mm3e_scene::n_lights() const {
    return low.blob.empty() ? 0u : reinterpret_cast<const TapeHeader*>(low.blob.data())->n_lights;
}

size_t mm3e_scene::device_bytes() const {
    size_t b = tape_cap + dyn_cap + buf.bytes() + (d_out ? pixels * sizeof(float4) : 0);
    for (const auto& p : low.payloads) b += p.bytes;
    return b;
}

const SpecKernels* mm3e_scene::spec_kernels() const { return spec ? &spec->kernels : nullptr; }

mm3e_scene::~mm3e_scene() {
    if (ctx) cudaSetDevice(ctx->device);
    spec.reset();
    cudaFree(d_tape);
    cudaFree(d_dyn_tape);
    for (void* p : d_payloads) cudaFree(p);
    cudaFree(d_kernel);
    cudaFree(d_out);
    buf.release();
    if (h_stage) cudaFreeHost(h_stage);
}

namespace {

// Upload the lowered tape (patching payload device addresses) into `*dst` (grown as needed).
int upload_tape(mm3e_scene* s, const LoweredScene& low, unsigned char** dst, size_t* cap, bool upload_payloads) {
    mm3e_ctx* c = s->ctx;
    cudaError_t e;
    if (upload_payloads) {
        for (void* p : s->d_payloads) cudaFree(p);
        s->d_payloads.clear();
        for (const auto& pl : low.payloads) {
            void* p = nullptr;
            e = cudaMalloc(&p, pl.bytes ? pl.bytes : 16);
            if (e != cudaSuccess) return cuda_fail(c, e, "payload allocation");
            e = cudaMemcpy(p, pl.host, pl.bytes, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cuda_fail(c, e, "payload upload");
            s->d_payloads.push_back(p);
        }
    }
    std::vector<unsigned char> blob = low.blob;
    for (size_t i = 0; i < low.payloads.size() && i < s->d_payloads.size(); ++i) {
        const void* addr = s->d_payloads[i];
        std::memcpy(blob.data() + low.payloads[i].patch_offset, &addr, sizeof(addr));
    }
    if (*cap < blob.size()) {
        cudaFree(*dst);
        *dst = nullptr;
        e = cudaMalloc(reinterpret_cast<void**>(dst), blob.size());
        if (e != cudaSuccess) return cuda_fail(c, e, "tape allocation");
        *cap = blob.size();
    }
    e = cudaMemcpyAsync(*dst, blob.data(), blob.size(), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "tape upload");
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "tape upload");
    return MM3E_OK;
}

// Frame buffers of the scene for the context's tile shape, allocated on the first frame (a
// scene that is only rendered through batches or the server holds just its tape). `host`
// also allocates the output framebuffer and pinned staging used by host-output calls.
int ensure_frame_buffers(mm3e_scene* s, bool host) {
    mm3e_ctx* c = s->ctx;
    cudaError_t e;
    uint32_t wlog = s->tuning().tile_wlog;
    size_t n = (size_t)s->low.width * s->low.height;
    size_t samples = slots_of(s->low.width, s->low.height, wlog) * s->low.aa * s->low.aa;
    if (n != s->pixels) {
        cudaFree(s->d_out);
        if (s->h_stage) cudaFreeHost(s->h_stage);
        s->d_out = nullptr;
        s->h_stage = nullptr;
        s->pixels = n;
    }
    if (host && n && !s->d_out) {
        e = cudaMalloc(reinterpret_cast<void**>(&s->d_out), n * sizeof(float4));
        if (e != cudaSuccess) return cuda_fail(c, e, "frame buffer allocation");
        e = cudaMallocHost(&s->h_stage, n * sizeof(float4));
        if (e != cudaSuccess) {
            cudaFree(s->d_out);
            s->d_out = nullptr;
            return cuda_fail(c, e, "pinned staging allocation");
        }
    }
    if (!s->buf.counters || s->buf_wlog != wlog || s->buf.cap < samples || s->buf.pixels < n ||
        s->buf.lights < s->n_lights() || s->buf.levels < s->low.bounces + 1) {
        e = s->buf.ensure(samples ? samples : 1, s->n_lights(), s->low.bounces + 1, n ? n : 1);
        if (e != cudaSuccess) return cuda_fail(c, e, "pass buffer allocation");
        s->buf_wlog = wlog;
    }
    return MM3E_OK;
}

int upload_post_kernel(mm3e_scene* s) {
    const mm3e_post& post = s->src.d.post;
    // the kernel is read only by blooming frames; without bloom a radius-1 kernel stands in
    uint32_t r = (post.bloom && post.bloom_intensity > 0.0f) ? post.bloom_radius : 1u;
    std::vector<float> k = gaussian_kernel(r);
    cudaFree(s->d_kernel);
    s->d_kernel = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&s->d_kernel), k.size() * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "bloom kernel allocation");
    e = cudaMemcpy(s->d_kernel, k.data(), k.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(s->ctx, e, "bloom kernel upload");
    s->bloom_radius = (uint32_t)(k.size() / 2);
    return MM3E_OK;
}

// Re-lower the scene from its host copy and upload tape + payloads.
int relower(mm3e_scene* s) {
    std::string err;
    LoweredScene low;
    int rc = lower_scene(s->src.d, nullptr, 0, low, err);
    if (rc) return fail(s->ctx, rc, err);
    s->low = std::move(low);
    s->spec.reset();  // compiled for the previous tape
    rc = upload_tape(s, s->low, &s->d_tape, &s->tape_cap, true);
    if (rc) return rc;
    return upload_post_kernel(s);
}

int check_status(mm3e_ctx* c, const uint32_t* d_status) {
    uint32_t st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "render");
    if (st & ST_TAPE_TIMEOUT) return fail(c, MM3E_ERR_TIMEOUT, "scene tape staging wait gave up");
    if (st & ST_TAPE_CORRUPT) return fail(c, MM3E_ERR_CUDA, "scene tape corrupt after staging");
    return MM3E_OK;
}

int check_status(mm3e_scene* s) { return check_status(s->ctx, s->buf.counters + (N_COUNTERS - 1)); }

#define CK(x)                                                   \
    do {                                                        \
        cudaError_t e_ = (x);                                   \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #x);     \
    } while (0)

// Single-job plan of one beauty frame of `s`.
PassPlan scene_plan(mm3e_scene* s, const unsigned char* tape, uint32_t tape_bytes, const mm3e_camera& cam,
                    uint32_t format, void* dout) {
    PassPlan p = plain_plan(s, cam, 0, 0, format, dout, s->buf_wlog);
    p.job0.tape = tape;
    p.tape_bytes = tape_bytes;
    return p;
}

// Pixel-centre march of job 0 (AOV / hits): hit records in the pass buffers, row-major slots.
int march_centers(mm3e_scene* s, const mm3e_camera* cam, const unsigned char* tape, uint32_t tape_bytes,
                  bool want_ao, LaunchLog* log, WaveArgs& a) {
    mm3e_ctx* c = s->ctx;
    uint32_t n = s->low.width * s->low.height;
    CK(cudaMemsetAsync(s->buf.counters, 0, N_COUNTERS * sizeof(uint32_t), c->stream));
    a = WaveArgs{};
    a.job0 = scene_job(s, tape, *cam, 0, 0, s->buf_wlog);
    a.tape_bytes = tape_bytes;
    a.cap = (uint32_t)s->buf.cap;
    a.lights_max = s->n_lights();
    a.tile_wlog = s->buf_wlog;
    a.grid_cap = (uint32_t)c->sm_count * 16u;
    a.status = s->buf.counters + (N_COUNTERS - 1);
    a.b.q_o = s->buf.qa_o;
    a.b.q_d = s->buf.qa_d;
    a.b.h_n = s->buf.h_n;
    a.b.h_m = s->buf.h_m;
    a.b.occ = s->buf.occ;
    a.src = SRC_CENTER;
    a.n_items = n;
    a.counter = s->buf.counters;
    a.wait_limit = c->wait_limit;
    a.wait_probe = c->wait_probe;
    const SpecKernels* sp = tape == s->d_tape ? s->spec_kernels() : nullptr;
    CK(launch_march(a, s->tuning(), c->stream, c->sm_count, log, sp));
    if (want_ao) CK(launch_ao(a, c->stream, log, sp));
    return MM3E_OK;
}

// Render into device memory `dout` (w*h float4 or uchar4). Asynchronous on the ctx stream.
// linear_only: beauty radiance into s->buf.hdr only (no post).
int render_to_device(mm3e_scene* s, const mm3e_camera* cam, const mm3e_dyn_sphere* dyn, size_t n_dyn, uint32_t format,
                     void* dout, bool linear_only, LaunchLog* log) {
    mm3e_ctx* c = s->ctx;
    const unsigned char* tape = s->d_tape;
    uint32_t tape_bytes = (uint32_t)s->low.blob.size();
    uint32_t mode = s->low.mode;
    {
        int rc = ensure_frame_buffers(s, false);
        if (rc) return rc;
    }
    if (n_dyn > 0) {
        std::string err;
        LoweredScene low;
        int rc = lower_scene(s->src.d, dyn, n_dyn, low, err);
        if (rc) return fail(c, rc, err);
        rc = upload_tape(s, low, &s->d_dyn_tape, &s->dyn_cap, false);
        if (rc) return rc;
        tape = s->d_dyn_tape;
        tape_bytes = (uint32_t)low.blob.size();
    }
    uint32_t w = s->low.width, h = s->low.height;
    if ((size_t)w * h == 0) return MM3E_OK;
    if (mode == MM3E_MODE_BEAUTY || linear_only) {
        PassPlan p = scene_plan(s, tape, tape_bytes, *cam, format, dout);
        if (n_dyn == 0) p.spec = s->spec_kernels();  // the specialised field is the scene's own tape
        p.post = !linear_only;
        CK(run_beauty(p, s->buf, s->tuning(), c->stream, c->sm_count, log));
        return MM3E_OK;
    }
    // The AO display value of every hit comes from the AO pass, which also writes the value of a
    // marcher without AO samples (1, march.rs:266), so it runs whenever the mode is AO.
    WaveArgs a;
    int rc = march_centers(s, cam, tape, tape_bytes, mode == MM3E_MODE_AO, log, a);
    if (rc) return rc;
    a.aov_mode = mode;
    float4* out = format == MM3E_FB_RGBA_F32 ? static_cast<float4*>(dout) : s->buf.hdr;
    CK(launch_aov(a, out, c->stream, log));
    if (format == MM3E_FB_RGBA8) CK(launch_pack_rgba8(s->buf.hdr, static_cast<uchar4*>(dout), (size_t)w * h, c->stream, log));
    return MM3E_OK;
}

}  // namespace

namespace {

bool finite3(const float* a) { return std::isfinite(a[0]) && std::isfinite(a[1]) && std::isfinite(a[2]); }

// Host f32 helpers (vec.rs / camera.rs constructors).
struct F3 {
    float x, y, z;
};
F3 f3(const float* a) { return F3{a[0], a[1], a[2]}; }
F3 add(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
F3 sub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 scl(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
float dotf(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
F3 crossf(F3 a, F3 o) { return F3{a.y * o.z - a.z * o.y, a.z * o.x - a.x * o.z, a.x * o.y - a.y * o.x}; }
F3 normf(F3 a) {
    float len = std::sqrt(dotf(a, a));
    return len > 1e-12f ? scl(a, 1.0f / len) : F3{0, 0, 0};
}
void put3(float* d, F3 v) {
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}
// Mat3::from_axis_angle (vec.rs:136-141)
void axis_angle(F3 axis, float angle, F3 cols[3]) {
    F3 k = normf(axis);
    float s = sinf(angle), c = cosf(angle);
    F3 es[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i) {
        F3 e = es[i];
        cols[i] = add(add(scl(e, c), scl(crossf(k, e), s)), scl(k, dotf(k, e) * (1.0f - c)));
    }
}
F3 mulv(const F3 m[3], F3 v) { return add(add(scl(m[0], v.x), scl(m[1], v.y)), scl(m[2], v.z)); }

}  // namespace

extern "C" {

int mm3e_abi_version(void) { return MM3E_ABI_VERSION; }

void mm3e_camera_look_at(const float eye[3], const float target[3], const float up_hint[3], float fov_y,
                         mm3e_camera* out) {
    F3 e = f3(eye);
    F3 fwd = normf(sub(f3(target), e));
    F3 right = normf(crossf(fwd, f3(up_hint)));
    F3 up = crossf(right, fwd);
    put3(out->eye, e);
    put3(out->forward, fwd);
    put3(out->right, right);
    put3(out->up, up);
    out->fov_scale = tanf(fov_y * 0.5f);
}

void mm3e_orbit_camera(const float target[3], float radius, float yaw, float pitch, float fov_y, mm3e_camera* out) {
    const float PI = 3.14159265358979323846f, TAU = 6.28318530717958647692f, FRAC_PI_2 = 1.57079632679489661923f;
    if (std::isfinite(yaw)) {  // wrap_orbit_yaw (lib.rs:1414-1420)
        float r = std::fmod(yaw + PI, TAU);
        if (r < 0.0f) r = r + std::fabs(TAU);
        yaw = r - PI;
    } else {
        yaw = 0.0f;
    }
    float lim = FRAC_PI_2 - 1.0e-4f;
    if (std::isfinite(pitch)) {
        if (pitch < -lim) pitch = -lim;
        if (pitch > lim) pitch = lim;
    } else {
        pitch = 0.0f;
    }
    radius = std::isfinite(radius) ? std::fmax(std::fabs(radius), 1.0e-4f) : 1.0f;
    if (std::isfinite(fov_y)) {
        if (fov_y < 1.0e-4f) fov_y = 1.0e-4f;
        if (fov_y > PI - 1.0e-4f) fov_y = PI - 1.0e-4f;
    } else {
        fov_y = 45.0f * (PI / 180.0f);
    }
    F3 t = f3(target);
    F3 eye = add(t, F3{radius * cosf(yaw) * cosf(pitch), radius * sinf(pitch), radius * sinf(yaw) * cosf(pitch)});
    float e[3] = {eye.x, eye.y, eye.z};
    const float up[3] = {0.0f, 1.0f, 0.0f};
    mm3e_camera_look_at(e, target, up, fov_y, out);
}

void mm3e_mat3_from_euler(float x, float y, float z, float out_cols[9]) {
    F3 rx[3], ry[3], rz[3], rxy[3], r[3];
    axis_angle(F3{1, 0, 0}, x, rx);
    axis_angle(F3{0, 1, 0}, y, ry);
    axis_angle(F3{0, 0, 1}, z, rz);
    for (int i = 0; i < 3; ++i) rxy[i] = mulv(rx, ry[i]);
    for (int i = 0; i < 3; ++i) r[i] = mulv(rxy, rz[i]);
    for (int i = 0; i < 3; ++i) put3(out_cols + 3 * i, r[i]);
}

void mm3e_quat_to_mat3(const float q_xyzw[4], float out_cols[9]) {
    float x = q_xyzw[0], y = q_xyzw[1], z = q_xyzw[2], w = q_xyzw[3];
    float n = std::sqrt(x * x + y * y + z * z + w * w);
    if (n > 1e-12f) {
        x = x / n;
        y = y / n;
        z = z / n;
        w = w / n;
    } else {
        x = y = z = 0.0f;
        w = 1.0f;
    }
    F3 c0{1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + z * w), 2.0f * (x * z - y * w)};
    F3 c1{2.0f * (x * y - z * w), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + x * w)};
    F3 c2{2.0f * (x * z + y * w), 2.0f * (y * z - x * w), 1.0f - 2.0f * (x * x + y * y)};
    put3(out_cols, c0);
    put3(out_cols + 3, c1);
    put3(out_cols + 6, c2);
}

void mm3e_light_directional(const float toward[3], const float color[3], mm3e_light* out) {
    put3(out->vec, normf(f3(toward)));
    std::memcpy(out->color, color, 12);
    out->directional = 1;
    out->radius = 0.0f;
}

int mm3e_scene_validate(const mm3e_scene_desc* desc, char* err, size_t err_len) {
    if (!desc) return MM3E_ERR_INVALID;
    std::string msg;
    int rc = validate_scene(*desc, msg);
    if (err && err_len) {
        std::strncpy(err, msg.c_str(), err_len - 1);
        err[err_len - 1] = 0;
    }
    return rc;
}

int mm3e_scene_tape_bytes(const mm3e_scene_desc* desc, size_t* out_bytes) {
    if (!desc || !out_bytes) return MM3E_ERR_INVALID;
    std::string msg;
    LoweredScene low;
    int rc = lower_scene(*desc, nullptr, 0, low, msg);
    if (rc) return rc;
    *out_bytes = low.blob.size();
    return MM3E_OK;
}

int mm3e_scene_tape(const mm3e_scene_desc* desc, void* out, size_t cap, size_t* len) {
    if (!desc) return MM3E_ERR_INVALID;
    std::string msg;
    LoweredScene low;
    int rc = lower_scene(*desc, nullptr, 0, low, msg);
    if (rc) return rc;
    if (len) *len = low.blob.size();
    if (out && cap) std::memcpy(out, low.blob.data(), low.blob.size() < cap ? low.blob.size() : cap);
    return MM3E_OK;
}

int mm3e_ctx_create(int device, mm3e_ctx** out) {
    if (!out) return MM3E_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return MM3E_ERR_CUDA;
    if (device < 0 || device >= count) return MM3E_ERR_INVALID;
    std::unique_ptr<mm3e_ctx> c(new mm3e_ctx());
    c->device = device;
    if ((e = cudaSetDevice(device)) != cudaSuccess) return MM3E_ERR_CUDA;
    if ((e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking)) != cudaSuccess) return MM3E_ERR_CUDA;
    c->stream = c->own_stream;
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&c->clock_khz, cudaDevAttrClockRate, device);
    int ats = 0;
    cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
    c->host_access = ats == 1;
    *out = c.release();
    return MM3E_OK;
}

void mm3e_ctx_destroy(mm3e_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->batch.reset();
    std::set<mm3e_scene*> live;
    live.swap(ctx->scenes);
    for (mm3e_scene* s : live) delete s;  // scenes left alive by the caller
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

const char* mm3e_last_error(const mm3e_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int mm3e_ctx_set_host_writes(mm3e_ctx* ctx, int enable, int* active) {
    if (!ctx) return MM3E_ERR_INVALID;
    ctx->host_writes = enable != 0;
    if (active) *active = ctx->host_access && ctx->host_writes ? 1 : 0;
    return MM3E_OK;
}

int mm3e_ctx_set_tape_wait(mm3e_ctx* ctx, uint32_t limit, int probe) {
    if (!ctx) return MM3E_ERR_INVALID;
    ctx->wait_limit = limit;
    ctx->wait_probe = probe ? 1u : 0u;
    return MM3E_OK;
}

int mm3e_ctx_sync(mm3e_ctx* ctx) {
    if (!ctx) return MM3E_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? MM3E_OK : cuda_fail(ctx, e, "sync");
}

int mm3e_ctx_set_stream(mm3e_ctx* ctx, void* cuda_stream) {
    if (!ctx) return MM3E_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set stream");
    ctx->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : ctx->own_stream;
    return MM3E_OK;
}

int mm3e_ctx_device_info(mm3e_ctx* ctx, int* sm_count, int* clock_khz) {
    if (!ctx) return MM3E_ERR_INVALID;
    if (sm_count) *sm_count = ctx->sm_count;
    if (clock_khz) *clock_khz = ctx->clock_khz;
    return MM3E_OK;
}

int mm3e_ctx_set_tuning(mm3e_ctx* ctx, const mm3e_tuning* t) {
    if (!ctx || !t) return MM3E_ERR_INVALID;
    if (t->block != 128 && t->block != 256) return fail(ctx, MM3E_ERR_INVALID, "block must be 128 or 256");
    if (t->tile_wlog > 5) return fail(ctx, MM3E_ERR_INVALID, "tile_wlog must be 0..5");
    if (t->unroll < 1 || t->unroll > 64) return fail(ctx, MM3E_ERR_INVALID, "unroll must be 1..64");
    if (t->min_blocks > 16) return fail(ctx, MM3E_ERR_INVALID, "min_blocks must be 0..16");
    cudaError_t e = cudaStreamSynchronize(ctx->stream);  // frames in flight keep their buffers
    if (e != cudaSuccess) return cuda_fail(ctx, e, "set tuning");
    ctx->tune.block = t->block;
    ctx->tune.tile_wlog = t->tile_wlog;
    ctx->tune.unroll = t->unroll;
    ctx->tune.min_blocks = t->min_blocks;
    return MM3E_OK;
}

int mm3e_ctx_get_tuning(mm3e_ctx* ctx, mm3e_tuning* t) {
    if (!ctx || !t) return MM3E_ERR_INVALID;
    t->block = ctx->tune.block;
    t->tile_wlog = ctx->tune.tile_wlog;
    t->unroll = ctx->tune.unroll;
    t->min_blocks = ctx->tune.min_blocks;
    return MM3E_OK;
}

int mm3e_ctx_set_profiling(mm3e_ctx* ctx, int enable) {
    if (!ctx) return MM3E_ERR_INVALID;
    ctx->prof.on = enable != 0;
    return MM3E_OK;
}

int mm3e_ctx_kernel_times(mm3e_ctx* ctx, mm3e_kernel_time* out, uint32_t cap, uint32_t* n_out) {
    if (!ctx) return MM3E_ERR_INVALID;
    static const char* names[KK_COUNT] = {"march", "ao", "shadow", "shade", "resolve", "post", "aov", "gi", "other",
                                          "march_refl", "ao_refl", "shadow_refl"};
    cudaError_t e = ctx->prof.collect(ctx->kk_ms, ctx->kk_launches);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel times");
    uint32_t n = 0;
    for (uint32_t k = 0; k < KK_COUNT; ++k) {
        if (!ctx->kk_launches[k]) continue;
        if (out && n < cap) {
            std::memset(&out[n], 0, sizeof(out[n]));
            std::strncpy(out[n].name, names[k], sizeof(out[n].name) - 1);
            out[n].launches = ctx->kk_launches[k];
            out[n].ms = ctx->kk_ms[k];
        }
        ++n;
    }
    for (uint32_t k = 0; k < KK_COUNT; ++k) {
        ctx->kk_ms[k] = 0.0;
        ctx->kk_launches[k] = 0;
    }
    if (n_out) *n_out = n;
    return MM3E_OK;
}

int mm3e_scene_compile(mm3e_ctx* ctx, const mm3e_scene_desc* desc, mm3e_scene** out) {
    if (!ctx || !desc || !out) return fail(ctx, MM3E_ERR_INVALID, "null argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    std::string err;
    int rc = validate_scene(*desc, err);
    if (rc) return fail(ctx, rc, err);
    std::unique_ptr<mm3e_scene> s(new mm3e_scene());
    s->ctx = ctx;
    s->src.assign(*desc);
    rc = relower(s.get());
    if (rc) return rc;
    *out = s.release();
    ctx->scenes.insert(*out);
    return MM3E_OK;
}

void mm3e_scene_destroy(mm3e_scene* scene) {
    if (!scene) return;
    if (scene->ctx) {
        if (!scene->ctx->scenes.erase(scene)) return;  // not a live scene of its context
        cudaStreamSynchronize(scene->ctx->stream);
    }
    delete scene;
}

int mm3e_scene_device_bytes(mm3e_scene* scene, size_t* out_bytes) {
    if (!scene || !out_bytes) return MM3E_ERR_INVALID;
    *out_bytes = scene->device_bytes();
    return MM3E_OK;
}

int mm3e_render(mm3e_scene* s, const mm3e_camera* camera, const mm3e_dyn_sphere* dyn, size_t n_dyn, uint32_t format,
                void* host_out, size_t out_bytes, mm3e_render_stats* stats) {
    if (!s || !camera) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    auto t0 = std::chrono::steady_clock::now();
    if (format > MM3E_FB_RGBA8) return fail(c, MM3E_ERR_INVALID, "unknown framebuffer format");
    if (n_dyn && !dyn) return fail(c, MM3E_ERR_INVALID, "null dynamic sphere array");
    size_t n = (size_t)s->low.width * s->low.height;
    size_t px = format == MM3E_FB_RGBA8 ? 4 : 16;
    if (n && (!host_out || out_bytes < n * px)) return fail(c, MM3E_ERR_INVALID, "output buffer too small");
    std::string err;
    int rc = validate_dynamic(s->src.d, dyn, n_dyn, err);
    if (rc) return fail(c, rc, err);
    cudaSetDevice(c->device);
    // On a host whose page tables the device shares, the post kernel stores the frame straight
    // into the caller's buffer over the coherent link: no staging copy, no host memcpy.
    const bool direct = n && c->host_access && c->host_writes && ((uintptr_t)host_out % (px == 4 ? 4u : 16u)) == 0;
    rc = ensure_frame_buffers(s, !direct);
    if (rc) return rc;
    LaunchLog log = c->prof.log();
    cudaEventRecord(c->ev0, c->stream);
    rc = render_to_device(s, camera, dyn, n_dyn, format, direct ? host_out : (void*)s->d_out, false, &log);
    if (rc) return rc;
    cudaEventRecord(c->ev1, c->stream);
    if (n && !direct) {
        cudaError_t e = cudaMemcpyAsync(s->h_stage, s->d_out, n * px, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "framebuffer download");
    }
    rc = check_status(s);
    if (rc) return rc;
    if (n && !direct) std::memcpy(host_out, s->h_stage, n * px);
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        stats->device_ms = ms;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->h2d_bytes = 0;
        stats->d2h_bytes = n * px;
        stats->kernel_launches = log.launches;
    }
    return MM3E_OK;
}

int mm3e_render_linear(mm3e_scene* s, const mm3e_camera* camera, float* host_rgb, size_t n_floats) {
    if (!s || !camera) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    size_t n = (size_t)s->low.width * s->low.height;
    if (n && (!host_rgb || n_floats < 3 * n)) return fail(c, MM3E_ERR_INVALID, "output buffer too small");
    cudaSetDevice(c->device);
    int rc = ensure_frame_buffers(s, true);
    if (rc) return rc;
    LaunchLog log = c->prof.log();
    rc = render_to_device(s, camera, nullptr, 0, MM3E_FB_RGBA_F32, nullptr, true, &log);
    if (rc) return rc;
    if (n) {
        cudaError_t e = cudaMemcpyAsync(s->h_stage, s->buf.hdr, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "HDR download");
    }
    rc = check_status(s);
    if (rc) return rc;
    const float* src = static_cast<const float*>(s->h_stage);
    for (size_t i = 0; i < n; ++i) {
        host_rgb[3 * i] = src[4 * i];
        host_rgb[3 * i + 1] = src[4 * i + 1];
        host_rgb[3 * i + 2] = src[4 * i + 2];
    }
    return MM3E_OK;
}

int mm3e_render_device(mm3e_scene* s, const mm3e_camera* camera, uint32_t format, void* device_out, size_t out_bytes) {
    if (!s || !camera) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    if (format > MM3E_FB_LINEAR_F32) return fail(c, MM3E_ERR_INVALID, "unknown framebuffer format");
    size_t n = (size_t)s->low.width * s->low.height;
    size_t px = format == MM3E_FB_RGBA8 ? 4 : 16;
    if (n && (!device_out || out_bytes < n * px)) return fail(c, MM3E_ERR_INVALID, "output buffer too small");
    cudaSetDevice(c->device);
    LaunchLog log = c->prof.log();
    if (format == MM3E_FB_LINEAR_F32) {
        if (s->low.mode != MM3E_MODE_BEAUTY) return fail(c, MM3E_ERR_INVALID, "linear output needs beauty mode");
        int rc = ensure_frame_buffers(s, false);
        if (rc) return rc;
        float4* keep = s->buf.hdr;
        s->buf.hdr = static_cast<float4*>(device_out);
        rc = render_to_device(s, camera, nullptr, 0, format, device_out, true, &log);
        s->buf.hdr = keep;
        return rc;
    }
    return render_to_device(s, camera, nullptr, 0, format, device_out, false, &log);
}

int mm3e_bake_gi(mm3e_scene* s, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t samples) {
    if (!s) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    cudaSetDevice(c->device);
    GiSetup g;
    if (!gi_setup(s->src.d, nx, ny, nz, samples, g)) return MM3E_OK;  // nothing bounded: GI unchanged
    uint64_t probes = (uint64_t)g.nx * g.ny * g.nz;
    uint64_t items = probes * 6 * g.dirs_per_face;
    if (items >= 0x7FFFFFFFull) return fail(c, MM3E_ERR_INVALID, "GI probe grid too large");
    cudaError_t e = cudaSuccess;
    PassBuffers w;
    e = w.ensure(items, 0, 1, 1);
    if (e != cudaSuccess) return cuda_fail(c, e, "GI bake allocation");
    float4 *d_dirs = nullptr, *d_rad = nullptr, *d_cubes = nullptr;
    e = cudaMalloc(reinterpret_cast<void**>(&d_dirs), g.dirs.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_rad), items * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_cubes), probes * 6 * sizeof(float4));
    auto cleanup = [&]() {
        cudaFree(d_dirs);
        cudaFree(d_rad);
        cudaFree(d_cubes);
        w.release();
    };
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(c, e, "GI bake allocation");
    }
    std::vector<float> cubes4(probes * 24);
    e = cudaMemcpyAsync(d_dirs, g.dirs.data(), g.dirs.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.counters, 0, N_COUNTERS * sizeof(uint32_t), c->stream);
    WaveArgs a{};
    a.job0.tape = s->d_tape;
    a.tape_bytes = (uint32_t)s->low.blob.size();
    a.status = w.counters + (N_COUNTERS - 1);
    a.counter = w.counters;
    a.src = SRC_GATHER;
    a.n_items = (uint32_t)items;
    a.cap = (uint32_t)items;
    a.b.q_o = w.qa_o;
    a.b.q_d = w.qa_d;
    a.b.h_n = w.h_n;
    a.b.h_m = w.h_m;
    std::memcpy(a.gi_lo, g.lo, 12);
    std::memcpy(a.gi_cell, g.cell, 12);
    a.gi_nx = g.nx;
    a.gi_ny = g.ny;
    a.gi_nz = g.nz;
    a.dirs_per_face = g.dirs_per_face;
    a.gather_dirs = d_dirs;
    LaunchLog log = c->prof.log();
    if (e == cudaSuccess) e = launch_march(a, c->tune, c->stream, c->sm_count, &log);
    if (e == cudaSuccess) e = launch_gather_shade(a, d_rad, c->stream, &log);
    if (e == cudaSuccess) e = launch_gi_reduce(d_rad, d_dirs, g.dirs_per_face, (uint32_t)probes, d_cubes, c->stream, &log);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(cubes4.data(), d_cubes, cubes4.size() * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    int rc = e == cudaSuccess ? check_status(c, w.counters + (N_COUNTERS - 1)) : cuda_fail(c, e, "GI bake");
    cleanup();
    if (rc) return rc;
    SceneCopy& sc = s->src;
    sc.has_gi = true;
    std::memcpy(sc.gi.min, g.lo, 12);
    std::memcpy(sc.gi.size, g.size, 12);
    sc.gi.nx = g.nx;
    sc.gi.ny = g.ny;
    sc.gi.nz = g.nz;
    sc.gi_cubes.assign(probes * 18, 0.0f);
    for (uint64_t p = 0; p < probes; ++p)
        for (int f = 0; f < 6; ++f)
            for (int k = 0; k < 3; ++k) sc.gi_cubes[p * 18 + f * 3 + k] = cubes4[p * 24 + f * 4 + k];
    sc.fix();
    return relower(s);
}

int mm3e_scene_get_gi(mm3e_scene* s, float min[3], float size[3], uint32_t dims[3], float* cubes, size_t n_floats) {
    if (!s) return MM3E_ERR_INVALID;
    const SceneCopy& sc = s->src;
    if (!sc.has_gi) return fail(s->ctx, MM3E_ERR_INVALID, "scene has no GI volume");
    if (min) std::memcpy(min, sc.gi.min, 12);
    if (size) std::memcpy(size, sc.gi.size, 12);
    if (dims) {
        dims[0] = sc.gi.nx;
        dims[1] = sc.gi.ny;
        dims[2] = sc.gi.nz;
    }
    if (cubes) {
        if (n_floats < sc.gi_cubes.size()) return fail(s->ctx, MM3E_ERR_INVALID, "GI buffer too small");
        std::memcpy(cubes, sc.gi_cubes.data(), sc.gi_cubes.size() * sizeof(float));
    }
    return MM3E_OK;
}

}  // extern "C"

// Copy hit records (normal xyz + t, material/NIL + steps) out and split them.
static int download_hits(mm3e_ctx* c, const PassBuffers& w, size_t n, float* t, uint32_t* mat, uint32_t* steps,
                         float* normal3) {
    std::vector<float4> hn(n);
    std::vector<uint2> hm(n);
    cudaError_t e = cudaMemcpyAsync(hn.data(), w.h_n, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), w.h_m, n * sizeof(uint2), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "hits download");
    int rc = check_status(c, w.counters + (N_COUNTERS - 1));
    if (rc) return rc;
    for (size_t i = 0; i < n; ++i) {
        t[i] = hn[i].w;
        mat[i] = hm[i].x;
        if (steps) steps[i] = hm[i].y;
        if (normal3) {
            normal3[3 * i] = hn[i].x;
            normal3[3 * i + 1] = hn[i].y;
            normal3[3 * i + 2] = hn[i].z;
        }
    }
    return MM3E_OK;
}

extern "C" {

int mm3e_render_hits(mm3e_scene* s, const mm3e_camera* camera, float* t, uint32_t* mat, uint32_t* steps,
                     float* normal3) {
    if (!s || !camera || !t || !mat) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    cudaSetDevice(c->device);
    size_t n = (size_t)s->low.width * s->low.height;
    if (n == 0) return MM3E_OK;
    WaveArgs a;
    LaunchLog log = c->prof.log();
    int rc = ensure_frame_buffers(s, false);
    if (rc) return rc;
    rc = march_centers(s, camera, s->d_tape, (uint32_t)s->low.blob.size(), false, &log, a);
    if (rc) return rc;
    return download_hits(c, s->buf, n, t, mat, steps, normal3);
}

int mm3e_march_rays(mm3e_scene* s, const float* rays6, size_t n, float* t, uint32_t* mat, uint32_t* steps) {
    if (!s || (n && (!rays6 || !t || !mat))) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    if (n >= 0x7FFFFFFFull) return fail(c, MM3E_ERR_INVALID, "too many rays");
    if (n == 0) return MM3E_OK;
    cudaSetDevice(c->device);
    PassBuffers w;
    cudaError_t e = w.ensure(n, 0, 1, 1);
    if (e != cudaSuccess) return cuda_fail(c, e, "ray buffer allocation");
    std::vector<float4> o(n), d(n);
    for (size_t i = 0; i < n; ++i) {
        o[i] = make_float4(rays6[6 * i], rays6[6 * i + 1], rays6[6 * i + 2], 0.0f);
        d[i] = make_float4(rays6[6 * i + 3], rays6[6 * i + 4], rays6[6 * i + 5], 0.0f);
    }
    e = cudaMemcpyAsync(w.qa_o, o.data(), n * sizeof(float4), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.qa_d, d.data(), n * sizeof(float4), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.counters, 0, N_COUNTERS * sizeof(uint32_t), c->stream);
    WaveArgs a{};
    a.job0.tape = s->d_tape;
    a.tape_bytes = (uint32_t)s->low.blob.size();
    a.status = w.counters + (N_COUNTERS - 1);
    a.counter = w.counters;
    a.src = SRC_QUEUE;
    a.n_items = (uint32_t)n;
    a.cap = (uint32_t)n;
    a.b.q_o = w.qa_o;
    a.b.q_d = w.qa_d;
    a.b.h_n = w.h_n;
    a.b.h_m = w.h_m;
    LaunchLog log = c->prof.log();
    if (e == cudaSuccess) e = launch_march(a, c->tune, c->stream, c->sm_count, &log);
    int rc = e == cudaSuccess ? download_hits(c, w, n, t, mat, steps, nullptr) : cuda_fail(c, e, "march rays");
    w.release();
    return rc;
}

int mm3e_field(mm3e_scene* s, const float* points3, size_t n, float* dist, uint32_t* mat) {
    if (!s || (n && (!points3 || !dist || !mat))) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    if (n == 0) return MM3E_OK;
    if (n >= 0xFFFFFFFFull) return fail(c, MM3E_ERR_INVALID, "too many points");
    cudaSetDevice(c->device);
    float *d_p = nullptr, *d_d = nullptr;
    uint32_t* d_m = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d_p), 12 * n);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_d), 4 * n);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_m), 4 * n);
    if (e != cudaSuccess) {
        cudaFree(d_p);
        cudaFree(d_d);
        cudaFree(d_m);
        return cuda_fail(c, e, "field allocation");
    }
    LaunchLog log = c->prof.log();
    e = cudaMemcpyAsync(d_p, points3, 12 * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_field(s->d_tape, d_p, (uint32_t)n, d_d, d_m, c->stream, &log);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dist, d_d, 4 * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(mat, d_m, 4 * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_p);
    cudaFree(d_d);
    cudaFree(d_m);
    return e == cudaSuccess ? MM3E_OK : cuda_fail(c, e, "field");
}

int mm3e_scene_specialize(mm3e_scene* s, int mode, double* compile_ms) {
    if (!s) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    if (compile_ms) *compile_ms = 0.0;
    if (mode < 0 || mode > 2) return fail(c, MM3E_ERR_INVALID, "mode must be 0 (off), 1 (auto) or 2 (always)");
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);  // frames in flight may use the old kernels
    if (e != cudaSuccess) return cuda_fail(c, e, "specialize");
    s->spec.reset();
    if (mode == 0) return MM3E_OK;
    if (mode == 1 && spec_size(s->low.blob).objects > SPEC_AUTO_MAX_OBJECTS) return MM3E_OK;  // interpreter is faster
    bool smem = s->low.blob.size() <= 96 * 1024;
    const TuneParams& t = s->tuning();
    uint32_t block = t.block, unroll = t.unroll;
    std::string src = spec_source(s->low.blob, block, unroll, smem, t.min_blocks);
    std::unique_ptr<SpecModule> m(new SpecModule());
    m->kernels.block = block;
    m->kernels.smem_tape = smem;
    std::string err = m->build(src, c->device, compile_ms);
    if (!err.empty() && err.compare(0, 4, "LOG:") != 0) return fail(c, MM3E_ERR_UNSUPPORTED, "scene specialisation: " + err);
    s->spec = std::move(m);
    return MM3E_OK;
}

int mm3e_scene_is_specialized(mm3e_scene* s) { return s && s->spec ? 1 : 0; }

// Launch-shape search for one scene's plain frames: each candidate is applied to the scene
// (specialised kernels recompiled for it), timed over `repeats` frames with CUDA events, and the
// fastest is kept as the scene's own tuning.
int mm3e_scene_autotune(mm3e_scene* s, const mm3e_camera* camera, int spec_mode, const mm3e_tuning* candidates,
                        uint32_t n_candidates, uint32_t repeats, mm3e_tuning* best, mm3e_tune_entry* report,
                        uint32_t report_cap, uint32_t* n_report) {
    if (!s || !camera || (n_candidates && !candidates)) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    if (spec_mode < 0 || spec_mode > 2) return fail(c, MM3E_ERR_INVALID, "spec_mode must be 0, 1 or 2");
    static const mm3e_tuning builtin[] = {{128, 3, 64, 0}, {128, 2, 64, 0}, {128, 4, 64, 0}, {256, 4, 64, 0},
                                          {256, 3, 64, 0}, {256, 3, 64, 3}, {128, 3, 64, 7}, {128, 3, 32, 0}};
    if (!n_candidates) {
        candidates = builtin;
        n_candidates = (uint32_t)(sizeof(builtin) / sizeof(builtin[0]));
    }
    for (uint32_t k = 0; k < n_candidates; ++k) {
        const mm3e_tuning& t = candidates[k];
        if ((t.block != 128 && t.block != 256) || t.tile_wlog > 5 || t.unroll < 1 || t.unroll > 64 || t.min_blocks > 16)
            return fail(c, MM3E_ERR_INVALID, "autotune candidate out of range (block 128/256, tile 0..5, unroll 1..64, min_blocks 0..16)");
    }
    if (repeats == 0) repeats = 5;
    if (n_report) *n_report = 0;
    cudaSetDevice(c->device);
    const bool had = s->own_tune;
    const TuneParams keep = s->tune;
    double best_ms = INFINITY;
    uint32_t best_k = 0;
    for (uint32_t k = 0; k < n_candidates; ++k) {
        const mm3e_tuning& t = candidates[k];
        s->tune = TuneParams{t.block, t.tile_wlog, t.unroll, t.min_blocks};
        s->own_tune = true;
        int rc = mm3e_scene_specialize(s, spec_mode, nullptr);
        if (rc == MM3E_OK) rc = ensure_frame_buffers(s, true);
        std::vector<float> ms;
        for (uint32_t r = 0; rc == MM3E_OK && r < repeats + 2; ++r) {
            LaunchLog log;
            cudaEventRecord(c->ev0, c->stream);
            rc = render_to_device(s, camera, nullptr, 0, MM3E_FB_RGBA8, (void*)s->d_out, false, &log);
            cudaEventRecord(c->ev1, c->stream);
            if (rc == MM3E_OK) rc = check_status(s);
            float f = 0.0f;
            if (rc == MM3E_OK && cudaEventElapsedTime(&f, c->ev0, c->ev1) == cudaSuccess && r >= 2) ms.push_back(f);
        }
        if (rc != MM3E_OK) {
            s->tune = keep;
            s->own_tune = had;
            mm3e_scene_specialize(s, spec_mode, nullptr);
            return rc;
        }
        std::sort(ms.begin(), ms.end());
        double med = ms.empty() ? INFINITY : ms[ms.size() / 2];
        if (report && k < report_cap) {
            report[k].tuning = t;
            report[k].device_ms = med;
            if (n_report) *n_report = k + 1;
        }
        if (med < best_ms) {
            best_ms = med;
            best_k = k;
        }
    }
    const mm3e_tuning& b = candidates[best_k];
    s->tune = TuneParams{b.block, b.tile_wlog, b.unroll, b.min_blocks};
    s->own_tune = true;
    if (best) *best = b;
    return mm3e_scene_specialize(s, spec_mode, nullptr);
}

int mm3e_scene_spec_source(const mm3e_scene_desc* desc, char* out, size_t cap, size_t* len) {
    if (!desc) return MM3E_ERR_INVALID;
    std::string msg;
    LoweredScene low;
    int rc = lower_scene(*desc, nullptr, 0, low, msg);
    if (rc) return rc;
    std::string src = spec_source(low.blob, 128, 1, low.blob.size() <= 96 * 1024, 0);
    if (len) *len = src.size();
    if (out && cap) {
        size_t n = src.size() < cap - 1 ? src.size() : cap - 1;
        std::memcpy(out, src.data(), n);
        out[n] = 0;
    }
    return MM3E_OK;
}

int mm3e_spec_compile_check(const mm3e_scene_desc* desc, char* err, size_t err_len, double* compile_ms) {
    if (!desc) return MM3E_ERR_INVALID;
    std::string msg;
    LoweredScene low;
    int rc = lower_scene(*desc, nullptr, 0, low, msg);
    if (rc) return rc;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<char> cubin;
    std::string e = spec_compile(spec_source(low.blob, 128, 1, low.blob.size() <= 96 * 1024, 0), cubin);
    if (compile_ms) *compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (err && err_len) {
        std::strncpy(err, e.c_str(), err_len - 1);
        err[err_len - 1] = 0;
    }
    return (e.empty() || e.compare(0, 4, "LOG:") == 0) ? MM3E_OK : MM3E_ERR_UNSUPPORTED;
}

int mm3e_render_film(mm3e_scene* s, const mm3e_camera* camera, float aperture_radius, float focus_distance,
                     float* beauty3, float* foreground3, float* alpha, float* depth, float* normals3,
                     uint32_t* material_ids) {
    if (!s || !camera) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    // Lens::validate (camera.rs:25-34)
    if (!std::isfinite(aperture_radius) || aperture_radius < 0.0f)
        return fail(c, MM3E_ERR_INVALID, "aperture_radius must be finite and nonnegative");
    if (!std::isfinite(focus_distance) || focus_distance <= 0.0f)
        return fail(c, MM3E_ERR_INVALID, "focus_distance must be finite and positive");
    size_t n = (size_t)s->low.width * s->low.height;
    if (n == 0) return MM3E_OK;
    cudaSetDevice(c->device);
    int rc = ensure_frame_buffers(s, true);
    if (rc) return rc;
    LaunchLog log = c->prof.log();
    PassPlan p = scene_plan(s, s->d_tape, (uint32_t)s->low.blob.size(), *camera, MM3E_FB_RGBA_F32, nullptr);
    p.spec = s->spec_kernels();
    p.post = false;
    p.film = true;
    p.job0.lens_radius = aperture_radius;
    p.job0.focus_distance = focus_distance;
    CK(run_beauty(p, s->buf, s->tuning(), c->stream, c->sm_count, &log));
    std::vector<float4> hdr(n), fg(n), hn(n), qd(n);
    std::vector<uint2> hm(n);
    CK(cudaMemcpyAsync(hdr.data(), s->buf.hdr, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(fg.data(), s->buf.fg, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    // geometric AOVs: the centre pinhole ray of every pixel (film.rs:111-116)
    WaveArgs a;
    rc = march_centers(s, camera, s->d_tape, (uint32_t)s->low.blob.size(), false, &log, a);
    if (rc) return rc;
    CK(cudaMemcpyAsync(hn.data(), s->buf.h_n, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(hm.data(), s->buf.h_m, n * sizeof(uint2), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(qd.data(), s->buf.qa_d, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    rc = check_status(s);
    if (rc) return rc;
    const float* eye = camera->eye;
    const float* fwd = camera->forward;
    for (size_t i = 0; i < n; ++i) {
        if (beauty3) {
            beauty3[3 * i] = hdr[i].x;
            beauty3[3 * i + 1] = hdr[i].y;
            beauty3[3 * i + 2] = hdr[i].z;
        }
        if (alpha) alpha[i] = hdr[i].w;
        if (foreground3) {
            foreground3[3 * i] = fg[i].x;
            foreground3[3 * i + 1] = fg[i].y;
            foreground3[3 * i + 2] = fg[i].z;
        }
        bool hit = hm[i].x != NIL;
        if (depth) {
            // (hit.pos - eye) . forward with hit.pos = eye + dir * t (Ray::at), in binary32
            float t = hn[i].w;
            float px = eye[0] + qd[i].x * t, py = eye[1] + qd[i].y * t, pz = eye[2] + qd[i].z * t;
            depth[i] = hit ? (px - eye[0]) * fwd[0] + (py - eye[1]) * fwd[1] + (pz - eye[2]) * fwd[2] : INFINITY;
        }
        if (normals3) {
            normals3[3 * i] = hit ? hn[i].x : 0.0f;
            normals3[3 * i + 1] = hit ? hn[i].y : 0.0f;
            normals3[3 * i + 2] = hit ? hn[i].z : 0.0f;
        }
        if (material_ids) material_ids[i] = hit ? hm[i].x : NIL;
    }
    return MM3E_OK;
}

// render_gbuffer: an aa-1 beauty frame without post, packed with its primary hits.
int mm3e_render_gbuffer(mm3e_scene* s, const mm3e_camera* camera, const float* movers4, uint32_t n_movers,
                        uint8_t* color4, float* depth, int32_t* obj) {
    if (!s || !camera || (n_movers && !movers4)) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    size_t n = (size_t)s->low.width * s->low.height;
    if (n == 0) return MM3E_OK;
    cudaSetDevice(c->device);
    int rc = ensure_frame_buffers(s, false);
    if (rc) return rc;
    CK(c->preview.ensure(n, n_movers, 0));
    PreviewBuffers& pv = c->preview;
    LaunchLog log = c->prof.log();
    PassPlan p = scene_plan(s, s->d_tape, (uint32_t)s->low.blob.size(), *camera, MM3E_FB_RGBA_F32, nullptr);
    p.job0.aa = 1;  // one pixel-centre sample (lib.rs:978)
    p.job0.spp = 1;
    p.job0.n_samples = p.job0.n_slots;
    p.n_samples = p.job0.n_samples;
    p.spec = s->spec_kernels();
    p.post = false;
    if (n_movers)
        CK(cudaMemcpyAsync(pv.mover, movers4, n_movers * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
    CK(run_beauty(p, s->buf, s->tuning(), c->stream, c->sm_count, &log));
    WaveArgs a{};
    a.job0 = p.job0;
    a.tile_wlog = s->buf_wlog;
    a.grid_cap = (uint32_t)c->sm_count * 16u;
    a.b.q_o = s->buf.qa_o;
    a.b.q_d = s->buf.qa_d;
    a.b.h_n = s->buf.h_n;
    a.b.h_m = s->buf.h_m;
    a.b.hdr = s->buf.hdr;
    CK(launch_gbuffer_pack(a, p.n_slots, pv.mover, n_movers, pv.color, pv.depth, pv.obj, c->stream, &log));
    if (color4) CK(cudaMemcpyAsync(color4, pv.color, n * sizeof(uchar4), cudaMemcpyDeviceToHost, c->stream));
    if (depth) CK(cudaMemcpyAsync(depth, pv.depth, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (obj) CK(cudaMemcpyAsync(obj, pv.obj, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    return check_status(s);
}

// reproject / reproject_hybrid: forward warp, then the row fill or the hole re-render.
int mm3e_reproject(mm3e_ctx* c, uint32_t w, uint32_t h, const mm3e_camera* prev_camera, const uint8_t* color4,
                   const float* depth, const int32_t* obj, const mm3e_camera* new_camera, const float* deltas3,
                   uint32_t n_deltas, mm3e_scene* hybrid, uint8_t* out4) {
    if (!c || !prev_camera || !new_camera) return MM3E_ERR_INVALID;
    size_t n = (size_t)w * h;
    if (n == 0) return MM3E_OK;
    if (!color4 || !depth || !obj || !out4 || (n_deltas && !deltas3)) return MM3E_ERR_INVALID;
    if (n > 0xFFFFFFFFull) return fail(c, MM3E_ERR_INVALID, "reprojected frame too large");
    if (hybrid && hybrid->ctx != c) return fail(c, MM3E_ERR_INVALID, "hybrid scene belongs to another context");
    cudaSetDevice(c->device);
    CK(c->preview.ensure(n, 0, n_deltas));
    PreviewBuffers& pv = c->preview;
    LaunchLog log = c->prof.log();
    CameraArgs prev{}, next{};
    fill_camera(prev, *prev_camera);
    fill_camera(next, *new_camera);
    CK(cudaMemcpyAsync(pv.color, color4, n * sizeof(uchar4), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(pv.depth, depth, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(pv.obj, obj, n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
    if (n_deltas) CK(cudaMemcpyAsync(pv.delta, deltas3, 3 * n_deltas * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(launch_warp(prev, next, w, h, pv.depth, pv.obj, pv.delta, n_deltas, pv.keys, pv.color, pv.out, pv.filled,
                   c->stream, &log));
    if (!hybrid) {
        CK(launch_row_fill(w, h, pv.out, pv.filled, c->stream, &log));
        CK(cudaMemcpyAsync(out4, pv.out, n * sizeof(uchar4), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return MM3E_OK;
    }
    mm3e_scene* s = hybrid;
    int rc = ensure_frame_buffers(s, false);
    if (rc) return rc;
    if (s->buf.cap < n) CK(s->buf.ensure(n, s->n_lights(), s->low.bounces + 1, s->buf.pixels));
    CK(cudaMemsetAsync(pv.count, 0, sizeof(uint32_t), c->stream));
    CK(launch_hole_rays(next, w, h, pv.filled, s->buf.qa_o, s->buf.qa_d, pv.hole_pix, pv.count,
                        (uint32_t)c->sm_count * 16u, c->stream, &log));
    PassPlan p = scene_plan(s, s->d_tape, (uint32_t)s->low.blob.size(), *new_camera, MM3E_FB_RGBA_F32, nullptr);
    p.queue0 = pv.count;
    p.n_samples = (uint32_t)n;  // capacity: every pixel a hole
    p.spec = s->spec_kernels();
    p.post = false;
    CK(run_beauty(p, s->buf, s->tuning(), c->stream, c->sm_count, &log));
    WaveArgs a{};
    a.job0 = p.job0;
    a.cap = (uint32_t)s->buf.cap;
    a.n_items = (uint32_t)n;
    a.grid_cap = (uint32_t)c->sm_count * 16u;
    a.b.lvl = s->buf.lvl;
    a.b.term = s->buf.term;
    CK(launch_hole_resolve(a, pv.count, pv.hole_pix, pv.out, c->stream, &log));
    CK(cudaMemcpyAsync(out4, pv.out, n * sizeof(uchar4), cudaMemcpyDeviceToHost, c->stream));
    return check_status(s);
}

// Allocation-free ray queries: the scratch lives in noalloc.cu's fixed __device__ array.
int mm3e_march_rays_noalloc(mm3e_scene* s, const float* d_rays6, size_t n, float* d_t, uint32_t* d_mat,
                            uint32_t* d_steps) {
    if (!s || (n && (!d_rays6 || !d_t || !d_mat))) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "mm3e_march_rays_noalloc: selecting the context's device");
    const char* what = "";
    // the launch shape of mm3e_march_rays (the context's), so both calls march identically
    int rc = noalloc_march_rays(s->d_tape, (uint32_t)s->low.blob.size(), c->device, c->sm_count, c->stream, c->tune,
                                d_rays6, n, d_t, d_mat, d_steps, &what);
    if (rc == 1) return fail(c, MM3E_ERR_INVALID, what);
    if (rc == 2) return fail(c, MM3E_ERR_CUDA, what);
    if (rc == 3) return fail(c, MM3E_ERR_TIMEOUT, what);
    return MM3E_OK;
}

}  // extern "C"
