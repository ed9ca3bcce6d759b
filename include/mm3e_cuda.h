/*
 * mm3e_cuda.h — C ABI of the GB300 (sm_103a) per-pixel SDF render path.
 *
 * This is the drop-in boundary for MM3E's CPU render call. A caller marshals its
 * `mm3e_orchestrator::Scene` into the flat POD `mm3e_scene_desc` below, compiles it once
 * into a device-resident scene tape, and renders per camera. The returned framebuffer is
 * the one the reference returns: straight-alpha RGBA f32 with alpha = 1 (or its RGBA8
 * quantisation, `Framebuffer::to_rgba8` over black).
 *
 * Reference interfaces each entry point replaces (paths inside the MM3E repository):
 *   mm3e_render            <- mm3e_orchestrator::render_with_threads_checked
 *                             (mm3e-orchestrator/src/lib.rs:866-871) and
 *                             mm3e_cpu_parallel::CpuParallelScene::try_render
 *                             (mm3e-cpu-parallel/src/lib.rs:50-65, dynamic spheres)
 *   mm3e_render_linear     <- render_linear_with_threads_checked (lib.rs:902-907)
 *   mm3e_scene_compile     <- CpuParallelRenderer::compile (mm3e-cpu-parallel/src/lib.rs:101)
 *                             and GpuRenderer::compile_checked (mm3e-gpu/src/lib.rs:138-285)
 *   mm3e_bake_gi           <- Scene::bake_gi_checked (mm3e-orchestrator/src/appearance.rs:193-200)
 *   mm3e_camera_look_at    <- Camera::look_at (mm3e-kit/src/camera.rs:50-55)
 *   mm3e_orbit_camera      <- orbit_camera (mm3e-orchestrator/src/lib.rs:1426-1435)
 *   mm3e_mat3_from_euler   <- Mat3::from_euler (mm3e-kit/src/vec.rs:144-149)
 *   mm3e_quat_to_mat3      <- Quat::to_mat3 (mm3e-kit/src/vec.rs:318-326)
 *   mm3e_light_directional <- Light::directional (mm3e-orchestrator/src/lib.rs:513-515)
 *   mm3e_scene_validate    <- Scene::validate_appearance + GPU codegen checks
 *                             (appearance.rs:250-269, mm3e-gpu/src/wgsl.rs:41-47,
 *                             mm3e-gpu/src/lib.rs:139-141, csg.rs:154-236)
 *   mm3e_last_error        <- the `Err(String)` of every checked reference call
 *   mm3e_render_film       <- film::render_film with a thin Lens (film.rs:63-224, camera.rs:25-102)
 *   mm3e_render_gbuffer    <- render_gbuffer_checked (mm3e-orchestrator/src/lib.rs:951-1039)
 *   mm3e_reproject         <- reproject::reproject (reproject.rs:118-146) and
 *                             reproject_hybrid (lib.rs:1040-1080)
 *   mm3e_bake_mesh_sdf     <- mesh::bake_sdf (mm3e-orchestrator/src/mesh.rs:262-336)
 *   mm3e_scene_parse_mm3e  <- scene_io::parse (mm3e-orchestrator/src/scene_io.rs:196-281)
 *   mm3e_scene_write_mm3e  <- scene_io::try_serialize (scene_io.rs:32-120)
 *   mm3e_volume_parse_sdfv <- SdfVolume::from_sdfv_bytes (mm3e-kit/src/volume.rs:140-176)
 *   mm3e_volume_write_sdfv <- SdfVolume::to_sdfv_bytes (volume.rs:119-137)
 *
 * Conventions: 0 = success, negative = error (message via mm3e_last_error). Contexts are not
 * thread-safe: use one context per host thread. All floats are IEEE binary32.
 */
#ifndef MM3E_CUDA_H
#define MM3E_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MM3E_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------------------------- */
enum {
    MM3E_OK = 0,
    MM3E_ERR_INVALID = -1,     /* bad scene / camera / argument (reference: Err(String)) */
    MM3E_ERR_UNSUPPORTED = -2, /* valid MM3E input this path does not render (UV maps, surfaces) */
    MM3E_ERR_CUDA = -3,        /* a CUDA runtime call failed */
    MM3E_ERR_NO_MEMORY = -4,   /* device or host allocation failed */
    MM3E_ERR_BUDGET = -5,      /* request refused by the HBM admission budget */
    MM3E_ERR_TIMEOUT = -6,     /* a bounded device-side wait gave up */
    MM3E_ERR_CANCELLED = -7,   /* request cancelled before completion */
    MM3E_ERR_BUSY = -8         /* no free slot right now (retry) */
};

/* ---- scene model (mirrors mm3e_orchestrator::{Prim, Combine, Modifiers, Object, Light,
 *      Scene}, mm3e_kit::{Material, Marcher}, post::Post) ---------------------------------- */

/* Prim (mm3e-orchestrator/src/lib.rs:157-212). Parameter packing in mm3e_object.params:
 *   SPHERE r | BOX hx hy hz | ROUND_BOX hx hy hz radius | TORUS major minor | CYLINDER h r |
 *   CAPSULE ax ay az bx by bz r | CONE r1 r2 h | ELLIPSOID rx ry rz | OCTAHEDRON s |
 *   HEX_PRISM r h | PLANE nx ny nz h | CSG (id = expression index) | VOLUME (id = volume index) */
enum {
    MM3E_PRIM_SPHERE = 0,
    MM3E_PRIM_BOX = 1,
    MM3E_PRIM_ROUND_BOX = 2,
    MM3E_PRIM_TORUS = 3,
    MM3E_PRIM_CYLINDER = 4,
    MM3E_PRIM_CAPSULE = 5,
    MM3E_PRIM_CONE = 6,
    MM3E_PRIM_ELLIPSOID = 7,
    MM3E_PRIM_OCTAHEDRON = 8,
    MM3E_PRIM_HEX_PRISM = 9,
    MM3E_PRIM_PLANE = 10,
    MM3E_PRIM_CSG = 11,
    MM3E_PRIM_VOLUME = 12,
    MM3E_PRIM_SURFACE = 13 /* native triangle shell: rejected, as the GPU twin does */
};

/* Combine (lib.rs:297-304) */
enum { MM3E_COMBINE_UNION = 0, MM3E_COMBINE_SMOOTH = 1, MM3E_COMBINE_SUBTRACT = 2 };

/* RenderMode (lib.rs:49-61) */
enum {
    MM3E_MODE_BEAUTY = 0,
    MM3E_MODE_NORMAL = 1,
    MM3E_MODE_DEPTH = 2,
    MM3E_MODE_AO = 3,
    MM3E_MODE_STEPS = 4,
    MM3E_MODE_ALBEDO = 5
};

/* Output framebuffer formats. */
enum {
    MM3E_FB_RGBA_F32 = 0, /* Framebuffer pixels: 4 x f32, straight alpha (= 1) */
    MM3E_FB_RGBA8 = 1,    /* Framebuffer::to_rgba8 over black: 4 x u8 */
    MM3E_FB_LINEAR_F32 = 2 /* render_linear radiance before post: 4 x f32 (rgb, 1); device output only */
};

/* Object (lib.rs:330-336) with Transform (vec.rs:165-169) and Modifiers (lib.rs:311-319). */
typedef struct mm3e_object {
    uint32_t prim;      /* MM3E_PRIM_* */
    uint32_t id;        /* CSG expression / volume index for CSG and VOLUME prims */
    uint32_t mat;       /* material index (reduced modulo the material count, as the reference) */
    uint32_t combine;   /* MM3E_COMBINE_* */
    float smooth_k;     /* Combine::Smooth(k) */
    float params[7];    /* primitive parameters, packed as documented above */
    float rot[9];       /* Mat3 columns: cols[0].xyz, cols[1].xyz, cols[2].xyz */
    float pos[3];
    float scale;
    uint32_t mirror;    /* bit 0 = x, bit 1 = y, bit 2 = z */
    float repeat[3];
    float twist;
    float bend;
    float elongate[3];
    float round;
    float onion;
} mm3e_object;

/* Material (mm3e-kit/src/color.rs:153-162) */
typedef struct mm3e_material {
    float albedo[3];
    float metallic;
    float specular;
    float roughness;
    float reflectivity;
    float emissive[3];
    uint32_t checker;
} mm3e_material;

/* Light (lib.rs:503-510). `vec` is the unit direction toward the light (directional) or the
 * light position (point / sphere). */
typedef struct mm3e_light {
    float vec[3];
    float color[3];
    uint32_t directional;
    float radius;
} mm3e_light;

/* Marcher (mm3e-kit/src/march.rs:42-79) */
typedef struct mm3e_marcher {
    uint32_t max_steps;
    float max_dist;
    float eps;
    float step_scale;
    uint32_t shadow_steps;
    uint32_t ao_samples;
    float lod_footprint;
    float subitize;
    uint32_t secant;
    float normal_h;
} mm3e_marcher;

/* Post (mm3e-orchestrator/src/post.rs:14-29) */
typedef struct mm3e_post {
    float exposure;
    uint32_t bloom;
    float bloom_threshold;
    float bloom_intensity;
    uint32_t bloom_radius;
} mm3e_post;

/* csg::Expr node (mm3e-kit/src/csg.rs:17-92), stored in an array; children by index.
 * kind: the 11 primitive kinds use MM3E_PRIM_* values 0..10 with `params` packed as for
 * objects; the operators below use `a`/`b` child indices. */
enum {
    MM3E_CSG_TRANSFORM = 100, /* child a, rot/pos/scale */
    MM3E_CSG_UNION = 101,     /* children a, b */
    MM3E_CSG_INTERSECT = 102,
    MM3E_CSG_SUBTRACT = 103,
    MM3E_CSG_SMOOTH_UNION = 104, /* params[0] = k */
    MM3E_CSG_OFFSET = 105,       /* child a, params[0] = distance */
    MM3E_CSG_SHELL = 106         /* child a, params[0] = thickness */
};
typedef struct mm3e_csg_node {
    uint32_t kind;
    uint32_t a;
    uint32_t b;
    uint32_t pad;
    float params[7];
    float rot[9];
    float pos[3];
    float scale;
} mm3e_csg_node;

/* SdfVolume (mm3e-kit/src/volume.rs:14-23); data row-major (k*ny + j)*nx + i. */
typedef struct mm3e_volume {
    uint32_t nx, ny, nz;
    float min[3];
    float cell[3];
    const float* data;
} mm3e_volume;

/* GiVolume (mm3e-orchestrator/src/gi.rs:17-23); cubes[((k*ny + j)*nx + i)*18 + face*3 + c],
 * faces +x, -x, +y, -y, +z, -z. */
typedef struct mm3e_gi {
    float min[3];
    float size[3];
    uint32_t nx, ny, nz;
    const float* cubes;
} mm3e_gi;

/* Scene (lib.rs:561-592). UV appearance bindings and native triangle surfaces are not part
 * of this path (the reference GPU twin rejects them too). */
typedef struct mm3e_scene_desc {
    uint32_t width;
    uint32_t height;
    const mm3e_object* objects;
    uint32_t n_objects;
    const mm3e_material* materials;
    uint32_t n_materials;
    const mm3e_light* lights;
    uint32_t n_lights;
    float sun_dir[3];
    float ambient[3];
    float sky_ambient[3];
    float fog[3];
    float fog_density;
    uint32_t aa;
    uint32_t bounces;
    uint32_t shadows;
    uint32_t ao;
    mm3e_marcher marcher;
    mm3e_post post;
    uint32_t mode;                  /* MM3E_MODE_* */
    const mm3e_gi* gi;              /* NULL = no baked GI */
    const mm3e_volume* volumes;
    uint32_t n_volumes;
    const mm3e_csg_node* csg_nodes; /* all expressions' nodes */
    uint32_t n_csg_nodes;
    const uint32_t* csg_roots;      /* root node index of expression i */
    uint32_t n_csgs;
} mm3e_scene_desc;

/* Camera (mm3e-kit/src/camera.rs:39-45) */
typedef struct mm3e_camera {
    float eye[3];
    float forward[3];
    float right[3];
    float up[3];
    float fov_scale; /* tan(fov_y / 2) */
} mm3e_camera;

/* DynSphere (mm3e-cpu-parallel/src/lib.rs:18-23) */
typedef struct mm3e_dyn_sphere {
    float pos[3];
    float radius;
    float albedo[3];
    float metallic;
} mm3e_dyn_sphere;

/* Per-render statistics (optional out-parameter). */
typedef struct mm3e_render_stats {
    double device_ms;      /* render + post kernels, CUDA events on the render stream */
    double total_ms;       /* host wall time of the call including copies */
    uint64_t h2d_bytes;
    uint64_t d2h_bytes;
    uint32_t kernel_launches;
} mm3e_render_stats;

typedef struct mm3e_ctx mm3e_ctx;
typedef struct mm3e_scene mm3e_scene;

/* ---- host-only helpers (no GPU needed) ---------------------------------------------------- */
int mm3e_abi_version(void);
void mm3e_camera_look_at(const float eye[3], const float target[3], const float up_hint[3], float fov_y,
                         mm3e_camera* out);
void mm3e_orbit_camera(const float target[3], float radius, float yaw, float pitch, float fov_y,
                       mm3e_camera* out);
void mm3e_mat3_from_euler(float x, float y, float z, float out_cols[9]);
void mm3e_quat_to_mat3(const float q_xyzw[4], float out_cols[9]);
void mm3e_light_directional(const float toward[3], const float color[3], mm3e_light* out);
/* Validates a scene description exactly as mm3e_scene_compile does, without a device. */
int mm3e_scene_validate(const mm3e_scene_desc* desc, char* err, size_t err_len);
/* Size in bytes of the lowered scene tape (host-side lowering, no device). */
int mm3e_scene_tape_bytes(const mm3e_scene_desc* desc, size_t* out_bytes);
/* The lowered scene tape itself (the bytes the device holds; host-side, no device): `len`
 * receives its size; up to `cap` bytes are copied to `out` (which may be NULL). For tools and
 * tests that evaluate the field on the host. */
int mm3e_scene_tape(const mm3e_scene_desc* desc, void* out, size_t cap, size_t* len);

/* ---- `.mm3e` text scenes (mm3e-orchestrator/src/scene_io.rs) -------------------------------- */
/* Parses a `.mm3e` document (scene_io::parse, scene_io.rs:196-281) into an owned scene
 * description and camera: same directives, defaults (Scene::new(640, 360), materials from the
 * file or one default) and validation, errors as "line N: ..." in `err`. Host only. */
typedef struct mm3e_parsed_scene mm3e_parsed_scene;
int mm3e_scene_parse_mm3e(const char* text, mm3e_parsed_scene** out, char* err, size_t err_len);
const mm3e_scene_desc* mm3e_parsed_scene_desc(const mm3e_parsed_scene* parsed);
int mm3e_parsed_scene_camera(const mm3e_parsed_scene* parsed, mm3e_camera* out);
void mm3e_parsed_scene_free(mm3e_parsed_scene* parsed);
/* scene_io::try_serialize (scene_io.rs:38-95): the `.mm3e` text of a scene + camera (numbers as
 * the shortest round-trip decimal). CSG / surface objects give MM3E_ERR_UNSUPPORTED with the
 * reference's message; volume objects become a comment. `out` may be NULL to query `len`. */
int mm3e_scene_write_mm3e(const mm3e_scene_desc* desc, const mm3e_camera* camera, char* out, size_t cap, size_t* len,
                          char* err, size_t err_len);

/* SdfVolume::from_sdfv_bytes (mm3e-kit/src/volume.rs:140-176): decodes an `.sdfv` buffer
 * ("MM3ESDF1", u32 nx ny nz, f32 min xyz, f32 cell xyz, then nx*ny*nz f32 samples, all
 * little-endian) into `out` (dims, min, cell; out->data = data) and, when `data` is not NULL,
 * its samples (capacity data_cap floats); *n_samples (may be NULL) receives nx*ny*nz. Errors:
 * MM3E_ERR_INVALID with the reference's message in err (truncation, magic, non-finite values,
 * overflow, length mismatch, SdfVolume::new's dims / cell rules). Host only; no GPU needed. */
int mm3e_volume_parse_sdfv(const uint8_t* bytes, size_t n, mm3e_volume* out, float* data, size_t data_cap,
                           size_t* n_samples, char* err, size_t err_len);
/* SdfVolume::to_sdfv_bytes (volume.rs:119-137): validates the volume (volume.rs:33-87) and
 * encodes it into out (capacity cap bytes; NULL: only *len). *len receives the encoded size. */
int mm3e_volume_write_sdfv(const mm3e_volume* volume, uint8_t* out, size_t cap, size_t* len, char* err,
                           size_t err_len);

/* ---- context ----------------------------------------------------------------------------- */
int mm3e_ctx_create(int device, mm3e_ctx** out);
/* Destroys the context and every scene still compiled on it (their handles become invalid). */
void mm3e_ctx_destroy(mm3e_ctx* ctx);
const char* mm3e_last_error(const mm3e_ctx* ctx);
int mm3e_ctx_sync(mm3e_ctx* ctx);
/* Run the context's work on a caller-owned cudaStream_t (NULL restores the context's own
 * stream); like cublasSetStream, for callers that order rendering with their own work. */
int mm3e_ctx_set_stream(mm3e_ctx* ctx, void* cuda_stream);
/* SM count and clock of the context's device (for roofline reporting). */
int mm3e_ctx_device_info(mm3e_ctx* ctx, int* sm_count, int* clock_khz);

/* Launch shape of the march and soft-shadow passes: threads per CTA (128 or 256), pixel tile
 * of 32 pixels 2^tile_wlog wide (tile_wlog 0..5; 3 = 8x4), and field samples per lane between
 * work refills (unroll 1..64, default 64; the tape interpreter's kernels round it down to 1, 16
 * or 64);
 * min_blocks (0..16) asks the compiler of scene-specialised
 * kernels to fit that many CTAs per SM in the register file (0: 8 CTAs of 128 or 4 of 256 for the
 * march and shadow kernels, the compiler's choice for the AO kernel). Results do not depend on it.
 * mm3e_autotune picks block / tile / unroll. */
typedef struct mm3e_tuning {
    uint32_t block, tile_wlog, unroll, min_blocks;
} mm3e_tuning;
int mm3e_ctx_set_tuning(mm3e_ctx* ctx, const mm3e_tuning* t);
int mm3e_ctx_get_tuning(mm3e_ctx* ctx, mm3e_tuning* t);

/* Per-kernel device time: when enabled, every pass is bracketed with CUDA events on the
 * context's stream (batched pass sequences then run without CUDA graphs).
 * mm3e_ctx_kernel_times waits for the recorded passes, writes one entry per kernel kind that
 * ran (march, ao, shadow, shade, resolve, post, aov, gi, other, march_refl, ao_refl,
 * shadow_refl: the *_refl kinds are the reflection levels' passes) and clears the totals. */
typedef struct mm3e_kernel_time {
    char name[16];
    uint32_t launches;
    double ms;
} mm3e_kernel_time;
int mm3e_ctx_set_profiling(mm3e_ctx* ctx, int enable);
/* Host framebuffers of mm3e_render: where the device reaches pageable host memory through the
 * host's page tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables, e.g. a Grace host on
 * NVLink-C2C), the post kernel writes the caller's buffer directly (default on); otherwise, or
 * with enable = 0 or an unaligned buffer (RGBA8: 4 bytes, RGBA f32: 16 bytes), the frame is
 * staged through pinned memory. Frames are identical either way. *active (may be NULL) receives
 * 1 when direct writes are in use. */
int mm3e_ctx_set_host_writes(mm3e_ctx* ctx, int enable, int* active);
/* The march and shadow kernels stage the scene tape into shared memory and wait for it on an
 * mbarrier with an iteration limit (the reference bounds every loop, march.rs:142,248; a device
 * wait here is bounded the same way): when the limit runs out the kernel records
 * MM3E_ERR_TIMEOUT for the call and returns, and the context stays usable. `limit` sets the
 * iterations of that wait for this context's plain calls (0: the default, 2^22). With probe = 1
 * the kernels issue no tape copy, so the wait runs to its limit with nothing in flight: a test of
 * the give-up path (every render then fails with MM3E_ERR_TIMEOUT until probe is set back to 0). */
int mm3e_ctx_set_tape_wait(mm3e_ctx* ctx, uint32_t limit, int probe);
int mm3e_ctx_kernel_times(mm3e_ctx* ctx, mm3e_kernel_time* out, uint32_t cap, uint32_t* n_out);

/* ---- scenes ------------------------------------------------------------------------------- */
/* Validates and lowers `desc` into a device-resident scene tape; `desc` may be freed after.
 * Beyond the reference's own rules, this path gives MM3E_ERR_UNSUPPORTED for aa > 16,
 * bounces > 7, a blooming scene's bloom_radius > 4096, CSG programs deeper than 16 values and
 * plain-union runs too large for its traversal stack. */
int mm3e_scene_compile(mm3e_ctx* ctx, const mm3e_scene_desc* desc, mm3e_scene** out);
void mm3e_scene_destroy(mm3e_scene* scene);
/* Device memory the compiled scene holds (tape, payloads, pass and frame buffers). */
int mm3e_scene_device_bytes(mm3e_scene* scene, size_t* out_bytes);

/* Render one frame of `scene` (scene->width x height, scene->mode) into host memory.
 * `dyn`/`n_dyn` append dynamic spheres exactly as CpuParallelScene::try_render does.
 * host_out must hold width*height*16 (RGBA_F32) or width*height*4 (RGBA8) bytes.
 * `stats` may be NULL. Blocking. */
int mm3e_render(mm3e_scene* scene, const mm3e_camera* camera, const mm3e_dyn_sphere* dyn, size_t n_dyn,
                uint32_t format, void* host_out, size_t out_bytes, mm3e_render_stats* stats);

/* Beauty radiance before post (render_linear): width*height*3 floats, row-major RGB. */
int mm3e_render_linear(mm3e_scene* scene, const mm3e_camera* camera, float* host_rgb, size_t n_floats);

/* Device-resident variant: writes into a device buffer on the context's stream (asynchronous;
 * call mm3e_ctx_sync before reading). Used by benchmarks and the batched/served forms. */
int mm3e_render_device(mm3e_scene* scene, const mm3e_camera* camera, uint32_t format, void* device_out,
                       size_t out_bytes);

/* Bake the GI ambient-cube probe volume on the GPU from the scene tape (Scene::bake_gi).
 * Replaces any GI the scene was compiled with. samples = rays per cube face (1 or 5). */
int mm3e_bake_gi(mm3e_scene* scene, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t samples);
/* Read back the scene's GI volume (e.g. after mm3e_bake_gi). `cubes` may be NULL to query dims. */
int mm3e_scene_get_gi(mm3e_scene* scene, float min[3], float size[3], uint32_t dims[3], float* cubes,
                      size_t n_floats);

/* ---- mesh -> SDF bake --------------------------------------------------------------------- */
/* An indexed triangle mesh (mesh.rs Mesh): positions xyz, triangles as 3 vertex indices. */
typedef struct mm3e_mesh {
    const float* positions;
    uint32_t n_positions;
    const uint32_t* triangles;
    uint32_t n_triangles;
} mm3e_mesh;
/* mesh::bake_sdf (mesh.rs:262-336) on the GPU: `resolution` samples along the longest padded
 * axis (clamped to 2..=512), `padding` > 0 around the mesh bounds. Fills out->nx/ny/nz, min,
 * cell; with `data` NULL only the grid is computed (query its size first). `data` receives
 * nx*ny*nz samples, (k*ny + j)*nx + i, in host memory (out->data is then set to it) or, with
 * data_on_device, in device memory. The samples equal the reference's: exact nearest-triangle
 * distance from the same BVH walk, sign from binary64 row-parity crossings. Errors carry the
 * reference's messages (no vertices / triangles, non-finite vertex, index out of range, bad
 * padding, only degenerate triangles). Blocking. */
int mm3e_bake_mesh_sdf(mm3e_ctx* ctx, const mm3e_mesh* mesh, uint32_t resolution, float padding, mm3e_volume* out,
                       float* data, size_t n_floats, int data_on_device);

/* ---- scene-specialised field (NVRTC) -------------------------------------------------------- */
/* Compiles, for this scene, march / shadow / AO kernels whose world field is generated from the
 * scene (the reference's GPU twin generates its `map` the same way, mm3e-gpu/src/wgsl.rs:277-319,
 * here with the CPU path's semantics): every object becomes a call of the library's own field
 * code on a constant copy of its record, every world-plan segment straight-line code with the
 * interpreter's fold, so frames are identical to the interpreted ones. Later mm3e_render /
 * mm3e_render_device / mm3e_render_linear / mm3e_render_hits calls of the scene use them (not
 * with dynamic spheres, not in batches). The launch shape is the context's tuning at this call.
 * mode 0 drops them; 2 always compiles; 1 (auto) compiles only scenes whose field inlines at
 * most 64 objects (the sizes measured faster than the shared-code interpreter; code size grows
 * with every object) and otherwise returns MM3E_OK leaving the interpreter. MM3E_ERR_UNSUPPORTED when
 * NVRTC cannot be loaded or compile fails. A GI bake (re-lowering) drops them. compile_ms may be
 * NULL. Blocking. */
int mm3e_scene_specialize(mm3e_scene* scene, int mode, double* compile_ms);
/* 1 when the scene renders with specialised kernels. */
int mm3e_scene_is_specialized(mm3e_scene* scene);
/* Host-only helpers (no device): the generated program of a scene description, and an NVRTC
 * compile of it to an sm_103a cubin (err receives the compiler log on failure). */
int mm3e_scene_spec_source(const mm3e_scene_desc* desc, char* out, size_t cap, size_t* len);
int mm3e_spec_compile_check(const mm3e_scene_desc* desc, char* err, size_t err_len, double* compile_ms);

/* ---- diagnostics: primary hits, arbitrary rays, field samples ------------------------------- */
/* Primary pinhole ray through every pixel centre (the ray RenderMode AOVs and the pinhole film
 * use, lib.rs:1179): hit distance t, material id (0xFFFFFFFF on a miss), march steps and the
 * hit normal (3 floats, zero on a miss). Any output pointer except `t` and `mat` may be NULL.
 * Replaces render_film's depth / matId AOVs for the pinhole lens (film.rs:89-146). */
int mm3e_render_hits(mm3e_scene* scene, const mm3e_camera* camera, float* t, uint32_t* mat, uint32_t* steps,
                     float* normal3);
/* render_film (mm3e-orchestrator/src/film.rs:63-139) with a thin lens (camera.rs Lens): per pixel
 * the scene-linear beauty (aa^2 samples through the lens; equal to mm3e_render_linear for a
 * zero aperture), the foreground premultiplied by coverage, the coverage alpha, and the centre
 * pinhole ray's geometric AOVs: camera-forward depth (+inf on a miss), world normal (zero on a
 * miss), material id (0xFFFFFFFF on a miss). Host outputs, width*height elements (3 floats for
 * beauty / foreground / normals); any may be NULL. Lens errors as Lens::validate. Blocking. */
int mm3e_render_film(mm3e_scene* scene, const mm3e_camera* camera, float aperture_radius, float focus_distance,
                     float* beauty3, float* foreground3, float* alpha, float* depth, float* normals3,
                     uint32_t* material_ids);
/* render_gbuffer (mm3e-orchestrator/src/lib.rs:951-1039): one pixel-centre sample per pixel, no
 * post pass. Per pixel (row-major, the scene's width*height): the display colour as RGBA8
 * (clamp01(gamma(aces(hdr * exposure))) * 255 + 0.5, alpha 255), the primary hit distance t
 * (+inf on a miss) and the index of the first mover (centre xyz, radius: 4 floats each, may be
 * NULL when n_movers is 0) whose sphere of radius + 0.05 holds the hit point (-1: none or a miss).
 * Host outputs; any may be NULL. Blocking. */
int mm3e_render_gbuffer(mm3e_scene* scene, const mm3e_camera* camera, const float* movers4, uint32_t n_movers,
                        uint8_t* color4, float* depth, int32_t* obj);
/* reproject::reproject (mm3e-orchestrator/src/reproject.rs:118-146) when hybrid_scene is NULL:
 * forward-warp a G-buffer frame (color4 / depth / obj as mm3e_render_gbuffer writes them, taken
 * at prev_camera, width*height) into new_camera, nearest point per target pixel, pixels of mover
 * k shifted by mover_deltas3[k] (xyz; k >= n_deltas: no shift), then fill each row's holes from
 * the last filled pixel to their left (the row's leading holes from its first filled pixel).
 * With hybrid_scene, reproject_hybrid (lib.rs:1040-1080): the holes are marched and shaded at
 * new_camera in hybrid_scene instead (display colour as mm3e_render_gbuffer). out4: width*height
 * RGBA8 (host). Blocking. */
int mm3e_reproject(mm3e_ctx* ctx, uint32_t width, uint32_t height, const mm3e_camera* prev_camera,
                   const uint8_t* color4, const float* depth, const int32_t* obj, const mm3e_camera* new_camera,
                   const float* mover_deltas3, uint32_t n_deltas, mm3e_scene* hybrid_scene, uint8_t* out4);
/* March `n` rays (origin xyz, unit direction xyz) with the scene's Marcher (march.rs:120-209). */
int mm3e_march_rays(mm3e_scene* scene, const float* rays6, size_t n, float* t, uint32_t* mat, uint32_t* steps);
/* World field (accelerated plan) at `n` points: Scene::field (lib.rs:715-717). */
int mm3e_field(mm3e_scene* scene, const float* points3, size_t n, float* dist, uint32_t* mat);

/* ---- batched rendering ---------------------------------------------------------------------- */
/* One frame of a batch: a compiled beauty-mode scene, a camera and an output. width/height 0
 * render at the scene's own size; otherwise the scene is rendered at width x height (the
 * reference renders any Scene at the size its caller sets). The frame goes to device_out
 * (device memory) or, when that is NULL, to host_out. */
typedef struct mm3e_job {
    mm3e_scene* scene;
    mm3e_camera camera;
    uint32_t width, height;
    uint32_t format;     /* MM3E_FB_RGBA8 or MM3E_FB_RGBA_F32 */
    void* device_out;
    void* host_out;
    size_t out_bytes;
} mm3e_job;

typedef struct mm3e_batch_config {
    uint64_t max_samples; /* samples (pixels x aa^2, tiles padded) per pass sequence; 0 = 2^24 */
    uint32_t use_graphs;  /* 1: replay each pass-sequence shape from a captured CUDA graph */
} mm3e_batch_config;

typedef struct mm3e_batch_stats {
    double device_ms;         /* CUDA events around the whole batch on the context's stream */
    double total_ms;          /* host wall time of the call */
    uint32_t sequences;       /* pass sequences (waves) run */
    uint32_t kernel_launches; /* kernels launched, graph kernel nodes included */
    uint32_t graph_launches;
    uint64_t samples;
    uint64_t h2d_bytes, d2h_bytes;
} mm3e_batch_stats;

int mm3e_batch_configure(mm3e_ctx* ctx, const mm3e_batch_config* cfg);
/* Renders every job; frames are identical to mm3e_render / mm3e_render_device of the same scene
 * and camera at the same size. Jobs are packed in order into pass sequences of at most
 * max_samples samples; each pass of a sequence is one launch over all its jobs. Blocking. */
int mm3e_render_batch(mm3e_ctx* ctx, const mm3e_job* jobs, size_t n, mm3e_batch_stats* stats);

/* Times every launch shape (block 128/256 x tile_wlog 2/3/4 x unroll 1/16/64) on `jobs` (each
 * rendered `repeats` times after a warm-up), keeps the fastest as the context's tuning and
 * reports the timings. */
typedef struct mm3e_tune_entry {
    mm3e_tuning tuning;
    double device_ms;
} mm3e_tune_entry;
int mm3e_autotune(mm3e_ctx* ctx, const mm3e_job* jobs, size_t n, uint32_t repeats, mm3e_tuning* best,
                  mm3e_tune_entry* report, uint32_t report_cap, uint32_t* n_report);
/* Launch-shape autotuning of one scene's plain frames (no reference counterpart: the tuning is
 * this library's). Each candidate (NULL / 0: a built-in set of block 128/256, tile and register
 * budgets) is applied to the scene, the scene re-specialised as `spec_mode` asks
 * (mm3e_scene_specialize modes), and `repeats` frames at `camera` timed with CUDA events (median);
 * the fastest becomes the scene's own tuning, used by its later frames instead of the context's,
 * and the scene is left specialised with it. Frames do not depend on the tuning. Blocking. */
int mm3e_scene_autotune(mm3e_scene* scene, const mm3e_camera* camera, int spec_mode, const mm3e_tuning* candidates,
                        uint32_t n_candidates, uint32_t repeats, mm3e_tuning* best, mm3e_tune_entry* report,
                        uint32_t report_cap, uint32_t* n_report);

/* ---- served form ----------------------------------------------------------------------------- */
/* A request loop with continuous batching: client threads submit requests, one worker thread
 * owns the device work. Scene tapes and payloads stay resident; requests are admitted against
 * an HBM budget and coalesced in arrival order into pass sequences on `max_inflight` slots
 * (own stream and buffers each), so requests arriving while others run start as soon as a
 * slot frees. While a server runs on a context, use that context only through the server. */
typedef struct mm3e_server mm3e_server;

typedef struct mm3e_server_config {
    uint64_t hbm_budget_bytes; /* resident scenes + slot buffers + admitted frames; 0 = 40 GiB */
    uint64_t max_samples;      /* samples per pass sequence; 0 = 2^23 */
    uint32_t max_inflight;     /* pass sequences on the GPU at once, 1..4; 0 = 2 */
    uint32_t use_graphs;       /* replay pass sequences from captured CUDA graphs */
    uint32_t plain;            /* 1: no coalescing; one request at a time through the per-frame
                                  launch sequence (the plain baseline) */
    uint32_t spec_workers;     /* host threads that compile scene-specialised kernels (NVRTC) for
                                  the resident scenes (mm3e_server_add_scene) in the background,
                                  at most 64 objects each; a scene's frames render with them once
                                  they are loaded, with the tape interpreter before (the same
                                  frames either way). 0: none. Not in plain mode. */
} mm3e_server_config;

typedef struct mm3e_request {
    uint32_t scene_id;                /* a resident scene (when new_scene is NULL) */
    const mm3e_scene_desc* new_scene; /* or a new scene: copied at submit, compiled, kept resident */
    const mm3e_mesh* mesh;            /* with new_scene: baked (mm3e_bake_mesh_sdf) into volume
                                         `mesh_volume` of the new scene before it is compiled;
                                         bakes are cached by mesh content */
    uint32_t mesh_volume, mesh_resolution;
    float mesh_padding;
    mm3e_camera camera;
    uint32_t width, height; /* 0: the scene's size */
    uint32_t format;        /* MM3E_FB_RGBA8 or MM3E_FB_RGBA_F32 */
    void* host_out;         /* receives the frame; must stay valid until the request completes */
    size_t out_bytes;
} mm3e_request;

typedef struct mm3e_request_result {
    int status;        /* MM3E_OK or the request's error code */
    uint32_t scene_id; /* scene rendered (new scenes are given an id) */
    double submit_ms;  /* server clock, ms: arrival (replay: the scheduled arrival) */
    double start_ms;   /* its pass sequence was launched */
    double done_ms;    /* its frame was in host memory */
} mm3e_request_result;

typedef struct mm3e_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t sequences, frames_in_sequences;
    uint64_t scenes_compiled, scenes_evicted, mesh_bakes, mesh_bake_hits;
    uint64_t admitted_bytes, peak_admitted_bytes, budget_bytes;
    uint64_t reserved_bytes; /* pass-sequence slot buffers, allocated when the server starts */
    uint64_t scenes_specialized; /* resident scenes whose specialised kernels are loaded */
    uint64_t spec_pending;       /* resident scenes whose specialised kernels are still compiling */
    uint64_t spec_frames;        /* frames rendered with specialised kernels */
} mm3e_server_stats;

int mm3e_server_create(mm3e_ctx* ctx, const mm3e_server_config* cfg, mm3e_server** out);
/* Compiles `desc` and keeps it resident; blocking. */
int mm3e_server_add_scene(mm3e_server* srv, const mm3e_scene_desc* desc, uint32_t* scene_id);
int mm3e_server_submit(mm3e_server* srv, const mm3e_request* req, uint64_t* ticket);
/* Waits up to timeout_ms (0: forever) for the request; MM3E_ERR_BUSY if it has not completed. */
int mm3e_server_wait(mm3e_server* srv, uint64_t ticket, uint32_t timeout_ms, mm3e_request_result* result);
int mm3e_server_get_stats(mm3e_server* srv, mm3e_server_stats* stats);
/* Open-loop load replay: a driver thread submits reqs[i] at arrival_s[i] seconds after the
 * call starts; returns when all completed. results[i] times are ms since the call started. */
int mm3e_server_replay(mm3e_server* srv, const mm3e_request* reqs, const double* arrival_s, size_t n,
                       mm3e_request_result* results);
/* Waits for every submitted request, then frees the server and its resident scenes. */
void mm3e_server_destroy(mm3e_server* srv);

/* ---- allocation-free ray queries --------------------------------------------------------- */
/* No counterpart in the reference: an addition for callers that cannot allocate device memory
 * while they query, e.g. a game or simulation loop casting picking / collision rays every frame
 * (cudaMalloc and cudaFree synchronise the device and can stall it for milliseconds) or a
 * service whose device memory is fully reserved up front by a pool or budget.
 * Marches `n` rays exactly as mm3e_march_rays does, but every pointer is DEVICE memory:
 * d_rays6 holds origin xyz + unit direction xyz per ray; d_t, d_mat (0xFFFFFFFF on a miss) and
 * d_steps (may be NULL) receive the results. The call allocates nothing: the ray queue and hit
 * records live in one fixed __device__ array (about 14.7 MB, held by every GPU that loads the
 * library until the process exits), so n is limited to 262144 rays per call (larger n returns
 * MM3E_ERR_INVALID). The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture. Every call shares the
 * array and overwrites it; calls that overlap on the GPU race on it, so serialise them.
 * The call runs on the context's stream (the caller's own stream after mm3e_ctx_set_stream):
 * d_rays6 must be complete before it runs, so either synchronise the work that writes it first
 * or write it on the stream given to mm3e_ctx_set_stream. cudaDeviceReset invalidates the cached
 * array address along with every context and scene of this library on that device.
 * Blocking: returns after the results are written. */
int mm3e_march_rays_noalloc(mm3e_scene* scene, const float* d_rays6, size_t n, float* d_t, uint32_t* d_mat,
                            uint32_t* d_steps);

#ifdef __cplusplus
}
#endif
#endif /* MM3E_CUDA_H */
