// capi.cpp — the C ABI (include/mm3e_cuda.h): contexts, compiled scenes and frame rendering.
//
// A context owns one CUDA stream on one device. A compiled scene owns its device tape, the
// uploaded payloads (SDF volume samples, GI probe cubes), the per-frame buffers (HDR, bloom
// scratch, output) and a pinned staging buffer for host copies, so a render call allocates
// nothing. Host-side arithmetic that mirrors Rust constructors is binary32 without
// contraction (this file is compiled with -ffp-contract=off).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "../../include/mm3e_cuda.h"
#include "kernels.h"
#include "lower.h"
#include "noalloc.h"

using namespace mm3e;

struct mm3e_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;      // stream all work is issued on
    cudaStream_t own_stream = nullptr;  // the context's own stream
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int sm_count = 0, clock_khz = 0;
    uint32_t* d_counter = nullptr;  // [0] work counter, [1] status word
    std::string err;
    std::set<mm3e_scene*> scenes;   // live scenes; destroyed with the context
};

namespace {

// Owned deep copy of a scene description (host), so dynamic spheres and GI bakes can
// re-lower the scene after the caller has released its arrays.
struct SceneCopy {
    mm3e_scene_desc d{};
    std::vector<mm3e_object> objects;
    std::vector<mm3e_material> materials;
    std::vector<mm3e_light> lights;
    std::vector<mm3e_volume> volumes;
    std::vector<std::vector<float>> volume_data;
    std::vector<mm3e_csg_node> csg_nodes;
    std::vector<uint32_t> csg_roots;
    bool has_gi = false;
    mm3e_gi gi{};
    std::vector<float> gi_cubes;

    void assign(const mm3e_scene_desc& s) {
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
    void fix() {
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
};

template <class T> T* dmalloc(size_t n, cudaError_t& e) {
    void* p = nullptr;
    e = cudaMalloc(&p, n * sizeof(T) + 16);
    return e == cudaSuccess ? static_cast<T*>(p) : nullptr;
}

int fail(mm3e_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}
int cuda_fail(mm3e_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? MM3E_ERR_NO_MEMORY : MM3E_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

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

}  // namespace

// Device buffers of the wavefront passes for up to `cap` rays (queues double-buffered).
struct WaveStore {
    size_t cap = 0, lights = 0, levels = 0;
    float4 *qa_o = nullptr, *qa_d = nullptr, *qb_o = nullptr, *qb_d = nullptr, *h_n = nullptr;
    uint2* h_m = nullptr;
    float *occ = nullptr, *shadow = nullptr;
    float4 *lvl = nullptr, *term = nullptr;
    void release() {
        void* ps[] = {qa_o, qa_d, qb_o, qb_d, h_n, h_m, occ, shadow, lvl, term};
        for (void* p : ps) cudaFree(p);
        *this = WaveStore();
    }
};

struct mm3e_scene {
    mm3e_ctx* ctx = nullptr;
    SceneCopy src;
    LoweredScene low;
    unsigned char* d_tape = nullptr;
    size_t tape_cap = 0;
    unsigned char* d_dyn_tape = nullptr;  // tape with dynamic spheres appended
    size_t dyn_cap = 0;
    std::vector<void*> d_payloads;        // same order as low.payloads
    float* d_kernel = nullptr;            // bloom weights
    uint32_t bloom_radius = 0;
    float4 *d_hdr = nullptr, *d_bright = nullptr, *d_blur = nullptr, *d_out = nullptr;
    void* h_stage = nullptr;              // pinned staging (w*h*16 bytes)
    size_t pixels = 0;
    WaveStore wave;                       // frame ray queues / hit records
    uint32_t* d_counters = nullptr;       // 64 words: work counters, queue lengths, status (63)

    ~mm3e_scene() {
        if (ctx) cudaSetDevice(ctx->device);
        cudaFree(d_tape);
        cudaFree(d_dyn_tape);
        for (void* p : d_payloads) cudaFree(p);
        cudaFree(d_kernel);
        cudaFree(d_hdr);
        cudaFree(d_bright);
        cudaFree(d_blur);
        cudaFree(d_out);
        cudaFree(d_counters);
        wave.release();
        if (h_stage) cudaFreeHost(h_stage);
    }
};

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

// Samples of one beauty frame: 8x4 pixel tiles (padding included) times aa^2.
size_t frame_samples(const LoweredScene& low) {
    size_t tiles = (size_t)((low.width + 7) / 8) * ((low.height + 3) / 4) * 32;
    return tiles * low.aa * low.aa;
}

int ensure_wave(mm3e_ctx* c, WaveStore& w, size_t cap, size_t lights, size_t levels) {
    if (cap <= w.cap && lights <= w.lights && levels <= w.levels) return MM3E_OK;
    w.release();
    cap = cap ? cap : 1;
    cudaError_t e = cudaSuccess;
    bool ok = (w.qa_o = dmalloc<float4>(cap, e)) && (w.qa_d = dmalloc<float4>(cap, e)) &&
              (w.qb_o = dmalloc<float4>(cap, e)) && (w.qb_d = dmalloc<float4>(cap, e)) &&
              (w.h_n = dmalloc<float4>(cap, e)) && (w.h_m = dmalloc<uint2>(cap, e)) &&
              (w.occ = dmalloc<float>(cap, e)) && (w.shadow = dmalloc<float>(cap * (lights ? lights : 1), e)) &&
              (w.lvl = dmalloc<float4>(cap * 2 * (levels ? levels : 1), e)) && (w.term = dmalloc<float4>(cap, e));
    if (!ok) {
        w.release();
        return cuda_fail(c, e, "ray queue allocation");
    }
    w.cap = cap;
    w.lights = lights;
    w.levels = levels;
    return MM3E_OK;
}

int ensure_frame_buffers(mm3e_scene* s) {
    mm3e_ctx* c = s->ctx;
    cudaError_t e;
    if (!s->d_counters) {
        s->d_counters = dmalloc<uint32_t>(64, e);
        if (!s->d_counters) return cuda_fail(c, e, "counter allocation");
    }
    size_t n = (size_t)s->low.width * s->low.height;
    if (n != s->pixels || (n && !s->d_hdr)) {
        cudaFree(s->d_hdr);
        cudaFree(s->d_bright);
        cudaFree(s->d_blur);
        cudaFree(s->d_out);
        if (s->h_stage) cudaFreeHost(s->h_stage);
        s->d_hdr = s->d_bright = s->d_blur = s->d_out = nullptr;
        s->h_stage = nullptr;
        s->pixels = n;
        if (n) {
            s->d_hdr = dmalloc<float4>(n, e);
            if (!s->d_hdr) return cuda_fail(c, e, "frame buffer allocation");
            s->d_bright = dmalloc<float4>(n, e);
            if (!s->d_bright) return cuda_fail(c, e, "frame buffer allocation");
            s->d_blur = dmalloc<float4>(n, e);
            if (!s->d_blur) return cuda_fail(c, e, "frame buffer allocation");
            s->d_out = dmalloc<float4>(n, e);
            if (!s->d_out) return cuda_fail(c, e, "frame buffer allocation");
            e = cudaMallocHost(&s->h_stage, n * sizeof(float4));
            if (e != cudaSuccess) return cuda_fail(c, e, "pinned staging allocation");
        }
    }
    size_t lights = s->low.blob.empty() ? 0 : reinterpret_cast<const TapeHeader*>(s->low.blob.data())->n_lights;
    return ensure_wave(c, s->wave, n ? frame_samples(s->low) : 0, lights, s->low.bounces);
}

int upload_post_kernel(mm3e_scene* s) {
    uint32_t r = s->src.d.post.bloom_radius;
    std::vector<float> k = gaussian_kernel(r);
    cudaFree(s->d_kernel);
    cudaError_t e;
    s->d_kernel = dmalloc<float>(k.size(), e);
    if (!s->d_kernel) return cuda_fail(s->ctx, e, "bloom kernel allocation");
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
    rc = upload_tape(s, s->low, &s->d_tape, &s->tape_cap, true);
    if (rc) return rc;
    rc = ensure_frame_buffers(s);
    if (rc) return rc;
    return upload_post_kernel(s);
}

void fill_camera(CameraArgs& a, const mm3e_camera& c) {
    std::memcpy(a.eye, c.eye, 12);
    std::memcpy(a.fwd, c.forward, 12);
    std::memcpy(a.right, c.right, 12);
    std::memcpy(a.up, c.up, 12);
    a.fov_scale = c.fov_scale;
}

int check_status(mm3e_scene* s) {
    mm3e_ctx* c = s->ctx;
    uint32_t st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, s->d_counters + 63, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "render");
    if (st & ST_TAPE_TIMEOUT) return fail(c, MM3E_ERR_TIMEOUT, "scene tape staging wait gave up");
    if (st & ST_TAPE_CORRUPT) return fail(c, MM3E_ERR_CUDA, "scene tape corrupt after staging");
    return MM3E_OK;
}

WaveArgs base_args(mm3e_scene* s, const unsigned char* tape, uint32_t tape_bytes) {
    WaveArgs a{};
    a.tape = tape;
    a.tape_bytes = tape_bytes;
    a.status = s->d_counters + 63;
    WaveStore& w = s->wave;
    a.b.q_o = w.qa_o;
    a.b.q_d = w.qa_d;
    a.b.h_n = w.h_n;
    a.b.h_m = w.h_m;
    a.b.occ = w.occ;
    a.b.shadow = w.shadow;
    a.b.nq_o = w.qb_o;
    a.b.nq_d = w.qb_d;
    a.b.lvl = w.lvl;
    a.b.term = w.term;
    a.b.hdr = s->d_hdr;
    return a;
}

#define CK(x)                                                   \
    do {                                                        \
        cudaError_t e_ = (x);                                   \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #x);     \
    } while (0)

// Beauty radiance of one frame into s->d_hdr: march / ao / shadow / shade per reflection
// level, then resolve (lib.rs:908-947, 1223-1360).
int render_beauty(mm3e_scene* s, const mm3e_camera* cam, const unsigned char* tape, uint32_t tape_bytes,
                  uint32_t* launches) {
    mm3e_ctx* c = s->ctx;
    const TapeHeader* h = reinterpret_cast<const TapeHeader*>(s->low.blob.data());
    uint32_t n = (uint32_t)frame_samples(s->low);
    CK(cudaMemsetAsync(s->d_counters, 0, 64 * sizeof(uint32_t), c->stream));
    WaveArgs a = base_args(s, tape, tape_bytes);
    fill_camera(a.cam, *cam);
    a.n_samples = n;
    bool ao = (h->flags & SF_AO) && h->ao_samples > 0;
    bool shadows = (h->flags & SF_SHADOWS) && h->shadow_steps > 0 && h->n_lights > 0;
    for (uint32_t level = 0; level <= s->low.bounces; ++level) {
        a.level = level;
        a.src = level == 0 ? SRC_SAMPLES : SRC_QUEUE;
        a.n_items = n;
        a.n_items_dev = level == 0 ? nullptr : s->d_counters + 4 * (level - 1) + 2;
        a.b.nq_count = s->d_counters + 4 * level + 2;
        a.counter = s->d_counters + 4 * level;
        CK(launch_march(a, c->stream, c->sm_count, launches));
        if (ao) CK(launch_ao(a, c->stream, launches));
        if (shadows) {
            a.counter = s->d_counters + 4 * level + 1;
            CK(launch_shadow(a, c->stream, c->sm_count, launches));
        }
        CK(launch_shade(a, c->stream, launches));
        std::swap(a.b.q_o, a.b.nq_o);
        std::swap(a.b.q_d, a.b.nq_d);
    }
    CK(launch_resolve(a, s->low.width, s->low.height, c->stream, launches));
    return MM3E_OK;
}

// Pixel-centre march (AOV / hits): hit records in the wave store, row-major slots.
int march_centers(mm3e_scene* s, const mm3e_camera* cam, const unsigned char* tape, uint32_t tape_bytes,
                  bool want_ao, uint32_t* launches, WaveArgs& a) {
    mm3e_ctx* c = s->ctx;
    uint32_t n = s->low.width * s->low.height;
    CK(cudaMemsetAsync(s->d_counters, 0, 64 * sizeof(uint32_t), c->stream));
    a = base_args(s, tape, tape_bytes);
    fill_camera(a.cam, *cam);
    a.src = SRC_CENTER;
    a.n_items = n;
    a.n_samples = n;
    a.counter = s->d_counters;
    CK(launch_march(a, c->stream, c->sm_count, launches));
    if (want_ao) CK(launch_ao(a, c->stream, launches));
    return MM3E_OK;
}

// Render into device memory `dout` (w*h float4 or uchar4). Asynchronous on the ctx stream.
int render_to_device(mm3e_scene* s, const mm3e_camera* cam, const mm3e_dyn_sphere* dyn, size_t n_dyn, uint32_t format,
                     void* dout, bool linear_only, uint32_t* launches) {
    mm3e_ctx* c = s->ctx;
    const unsigned char* tape = s->d_tape;
    uint32_t tape_bytes = (uint32_t)s->low.blob.size();
    uint32_t mode = s->low.mode;
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
        int rc = render_beauty(s, cam, tape, tape_bytes, launches);
        if (rc) return rc;
        if (linear_only) return MM3E_OK;
        PostArgs p{};
        p.hdr = s->d_hdr;
        p.bright = s->d_bright;
        p.blur_h = s->d_blur;
        p.kernel_w = s->d_kernel;
        p.radius = s->bloom_radius;
        p.width = w;
        p.height = h;
        const mm3e_post& post = s->src.d.post;
        p.bloom = post.bloom && post.bloom_intensity > 0.0f;
        p.threshold = post.bloom_threshold;
        p.intensity = post.bloom_intensity;
        p.exposure = post.exposure;
        p.format = (int)format;
        p.out = dout;
        CK(launch_post(p, c->stream, launches));
        return MM3E_OK;
    }
    const TapeHeader* th = reinterpret_cast<const TapeHeader*>(s->low.blob.data());
    WaveArgs a;
    int rc = march_centers(s, cam, tape, tape_bytes, mode == MM3E_MODE_AO && th->ao_samples > 0, launches, a);
    if (rc) return rc;
    a.aov_mode = mode;
    float4* out = format == MM3E_FB_RGBA_F32 ? static_cast<float4*>(dout) : s->d_hdr;
    CK(launch_aov(a, w, h, out, c->stream, launches));
    if (format == MM3E_FB_RGBA8) CK(launch_pack_rgba8(s->d_hdr, static_cast<uchar4*>(dout), (size_t)w * h, c->stream, launches));
    return MM3E_OK;
}

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
    if ((e = cudaMalloc(&c->d_counter, 4 * sizeof(uint32_t))) != cudaSuccess) return MM3E_ERR_NO_MEMORY;
    *out = c.release();
    return MM3E_OK;
}

void mm3e_ctx_destroy(mm3e_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    std::set<mm3e_scene*> live;
    live.swap(ctx->scenes);
    for (mm3e_scene* s : live) delete s;  // scenes left alive by the caller
    cudaFree(ctx->d_counter);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

const char* mm3e_last_error(const mm3e_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

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
    uint32_t launches = 0;
    cudaEventRecord(c->ev0, c->stream);
    rc = render_to_device(s, camera, dyn, n_dyn, format, s->d_out == nullptr ? nullptr : (void*)s->d_out, false,
                          &launches);
    if (rc) return rc;
    // AOV RGBA f32 writes straight into d_out; beauty post writes into d_out too.
    cudaEventRecord(c->ev1, c->stream);
    if (n) {
        cudaError_t e = cudaMemcpyAsync(s->h_stage, s->d_out, n * px, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "framebuffer download");
    }
    rc = check_status(s);
    if (rc) return rc;
    if (n) std::memcpy(host_out, s->h_stage, n * px);
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        stats->device_ms = ms;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->h2d_bytes = 0;
        stats->d2h_bytes = n * px;
        stats->kernel_launches = launches;
    }
    return MM3E_OK;
}

int mm3e_render_linear(mm3e_scene* s, const mm3e_camera* camera, float* host_rgb, size_t n_floats) {
    if (!s || !camera) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    size_t n = (size_t)s->low.width * s->low.height;
    if (n && (!host_rgb || n_floats < 3 * n)) return fail(c, MM3E_ERR_INVALID, "output buffer too small");
    cudaSetDevice(c->device);
    uint32_t launches = 0;
    int rc = render_to_device(s, camera, nullptr, 0, MM3E_FB_RGBA_F32, nullptr, true, &launches);
    if (rc) return rc;
    if (n) {
        cudaError_t e = cudaMemcpyAsync(s->h_stage, s->d_hdr, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
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
    if (format == MM3E_FB_LINEAR_F32) {
        if (s->low.mode != MM3E_MODE_BEAUTY) return fail(c, MM3E_ERR_INVALID, "linear output needs beauty mode");
        float4* keep = s->d_hdr;
        s->d_hdr = static_cast<float4*>(device_out);
        int rc = render_to_device(s, camera, nullptr, 0, format, device_out, true, nullptr);
        s->d_hdr = keep;
        return rc;
    }
    return render_to_device(s, camera, nullptr, 0, format, device_out, false, nullptr);
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
    WaveStore w;
    int rc = ensure_wave(c, w, items, 0, 0);
    if (rc) return rc;
    float4* d_dirs = dmalloc<float4>(g.dirs.size() / 4, e);
    float4* d_rad = d_dirs ? dmalloc<float4>(items, e) : nullptr;
    float4* d_cubes = d_rad ? dmalloc<float4>(probes * 6, e) : nullptr;
    auto cleanup = [&]() {
        cudaFree(d_dirs);
        cudaFree(d_rad);
        cudaFree(d_cubes);
        w.release();
    };
    if (!d_cubes) {
        cleanup();
        return cuda_fail(c, e, "GI bake allocation");
    }
    std::vector<float> cubes4(probes * 24);
    e = cudaMemcpyAsync(d_dirs, g.dirs.data(), g.dirs.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_counters, 0, 64 * sizeof(uint32_t), c->stream);
    WaveArgs a{};
    a.tape = s->d_tape;
    a.tape_bytes = (uint32_t)s->low.blob.size();
    a.status = s->d_counters + 63;
    a.counter = s->d_counters;
    a.src = SRC_GATHER;
    a.n_items = (uint32_t)items;
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
    if (e == cudaSuccess) e = launch_march(a, c->stream, c->sm_count, nullptr);
    if (e == cudaSuccess) e = launch_gather_shade(a, d_rad, c->stream, nullptr);
    if (e == cudaSuccess) e = launch_gi_reduce(d_rad, d_dirs, g.dirs_per_face, (uint32_t)probes, d_cubes, c->stream, nullptr);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(cubes4.data(), d_cubes, cubes4.size() * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    rc = e == cudaSuccess ? check_status(s) : cuda_fail(c, e, "GI bake");
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

// Copy hit records (normal xyz + t, material/NIL + steps) out and split them.
static int download_hits(mm3e_scene* s, const WaveStore& w, size_t n, float* t, uint32_t* mat, uint32_t* steps,
                         float* normal3) {
    mm3e_ctx* c = s->ctx;
    std::vector<float4> hn(n);
    std::vector<uint2> hm(n);
    cudaError_t e = cudaMemcpyAsync(hn.data(), w.h_n, n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hm.data(), w.h_m, n * sizeof(uint2), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "hits download");
    int rc = check_status(s);
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

int mm3e_render_hits(mm3e_scene* s, const mm3e_camera* camera, float* t, uint32_t* mat, uint32_t* steps,
                     float* normal3) {
    if (!s || !camera || !t || !mat) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    cudaSetDevice(c->device);
    size_t n = (size_t)s->low.width * s->low.height;
    if (n == 0) return MM3E_OK;
    WaveArgs a;
    int rc = march_centers(s, camera, s->d_tape, (uint32_t)s->low.blob.size(), false, nullptr, a);
    if (rc) return rc;
    return download_hits(s, s->wave, n, t, mat, steps, normal3);
}

int mm3e_march_rays(mm3e_scene* s, const float* rays6, size_t n, float* t, uint32_t* mat, uint32_t* steps) {
    if (!s || (n && (!rays6 || !t || !mat))) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    if (n >= 0x7FFFFFFFull) return fail(c, MM3E_ERR_INVALID, "too many rays");
    if (n == 0) return MM3E_OK;
    cudaSetDevice(c->device);
    WaveStore w;
    int rc = ensure_wave(c, w, n, 0, 0);
    if (rc) return rc;
    std::vector<float4> o(n), d(n);
    for (size_t i = 0; i < n; ++i) {
        o[i] = make_float4(rays6[6 * i], rays6[6 * i + 1], rays6[6 * i + 2], 0.0f);
        d[i] = make_float4(rays6[6 * i + 3], rays6[6 * i + 4], rays6[6 * i + 5], 0.0f);
    }
    cudaError_t e = cudaMemcpyAsync(w.qa_o, o.data(), n * sizeof(float4), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.qa_d, d.data(), n * sizeof(float4), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_counters, 0, 64 * sizeof(uint32_t), c->stream);
    WaveArgs a{};
    a.tape = s->d_tape;
    a.tape_bytes = (uint32_t)s->low.blob.size();
    a.status = s->d_counters + 63;
    a.counter = s->d_counters;
    a.src = SRC_QUEUE;
    a.n_items = (uint32_t)n;
    a.b.q_o = w.qa_o;
    a.b.q_d = w.qa_d;
    a.b.h_n = w.h_n;
    a.b.h_m = w.h_m;
    if (e == cudaSuccess) e = launch_march(a, c->stream, c->sm_count, nullptr);
    rc = e == cudaSuccess ? download_hits(s, w, n, t, mat, steps, nullptr) : cuda_fail(c, e, "march rays");
    w.release();
    return rc;
}

int mm3e_field(mm3e_scene* s, const float* points3, size_t n, float* dist, uint32_t* mat) {
    if (!s || (n && (!points3 || !dist || !mat))) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    if (n == 0) return MM3E_OK;
    if (n >= 0xFFFFFFFFull) return fail(c, MM3E_ERR_INVALID, "too many points");
    cudaSetDevice(c->device);
    cudaError_t e;
    float* d_p = dmalloc<float>(3 * n, e);
    float* d_d = d_p ? dmalloc<float>(n, e) : nullptr;
    uint32_t* d_m = d_d ? dmalloc<uint32_t>(n, e) : nullptr;
    if (!d_m) {
        cudaFree(d_p);
        cudaFree(d_d);
        return cuda_fail(c, e, "field allocation");
    }
    cudaMemcpyAsync(d_p, points3, 12 * n, cudaMemcpyHostToDevice, c->stream);
    e = launch_field(s->d_tape, (uint32_t)s->low.blob.size(), d_p, (uint32_t)n, d_d, d_m, c->stream, nullptr);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dist, d_d, 4 * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(mat, d_m, 4 * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_p);
    cudaFree(d_d);
    cudaFree(d_m);
    return e == cudaSuccess ? MM3E_OK : cuda_fail(c, e, "field");
}

// Allocation-free ray queries: the scratch lives in noalloc.cu's fixed __device__ array.
int mm3e_march_rays_noalloc(mm3e_scene* s, const float* d_rays6, size_t n, float* d_t, uint32_t* d_mat,
                            uint32_t* d_steps) {
    if (!s || (n && (!d_rays6 || !d_t || !d_mat))) return MM3E_ERR_INVALID;
    mm3e_ctx* c = s->ctx;
    cudaSetDevice(c->device);
    const char* what = "";
    int rc = noalloc_march_rays(s->d_tape, (uint32_t)s->low.blob.size(), c->device, c->sm_count, c->stream, d_rays6, n,
                                d_t, d_mat, d_steps, &what);
    if (rc == 1) return fail(c, MM3E_ERR_INVALID, what);
    if (rc == 2) return fail(c, MM3E_ERR_CUDA, what);
    if (rc == 3) return fail(c, MM3E_ERR_TIMEOUT, what);
    return MM3E_OK;
}

}  // extern "C"
