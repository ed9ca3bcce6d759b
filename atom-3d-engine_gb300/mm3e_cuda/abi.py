"""ctypes mirror of include/mm3e_cuda.h (the C ABI of the GB300 SDF render path)."""
import ctypes as C

ABI_VERSION = 2

OK = 0
ERR_INVALID = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_NO_MEMORY = -4
ERR_BUDGET = -5
ERR_TIMEOUT = -6
ERR_CANCELLED = -7
ERR_BUSY = -8

PRIM_SPHERE, PRIM_BOX, PRIM_ROUND_BOX, PRIM_TORUS, PRIM_CYLINDER, PRIM_CAPSULE, PRIM_CONE, \
    PRIM_ELLIPSOID, PRIM_OCTAHEDRON, PRIM_HEX_PRISM, PRIM_PLANE, PRIM_CSG, PRIM_VOLUME, PRIM_SURFACE = range(14)
COMBINE_UNION, COMBINE_SMOOTH, COMBINE_SUBTRACT = range(3)
MODE_BEAUTY, MODE_NORMAL, MODE_DEPTH, MODE_AO, MODE_STEPS, MODE_ALBEDO = range(6)
FB_RGBA_F32, FB_RGBA8, FB_LINEAR_F32 = range(3)
CSG_TRANSFORM, CSG_UNION, CSG_INTERSECT, CSG_SUBTRACT, CSG_SMOOTH_UNION, CSG_OFFSET, CSG_SHELL = range(100, 107)

F3 = C.c_float * 3


class Object(C.Structure):
    _fields_ = [("prim", C.c_uint32), ("id", C.c_uint32), ("mat", C.c_uint32), ("combine", C.c_uint32),
                ("smooth_k", C.c_float), ("params", C.c_float * 7), ("rot", C.c_float * 9), ("pos", F3),
                ("scale", C.c_float), ("mirror", C.c_uint32), ("repeat", F3), ("twist", C.c_float),
                ("bend", C.c_float), ("elongate", F3), ("round", C.c_float), ("onion", C.c_float)]


class Material(C.Structure):
    _fields_ = [("albedo", F3), ("metallic", C.c_float), ("specular", C.c_float), ("roughness", C.c_float),
                ("reflectivity", C.c_float), ("emissive", F3), ("checker", C.c_uint32)]


class Light(C.Structure):
    _fields_ = [("vec", F3), ("color", F3), ("directional", C.c_uint32), ("radius", C.c_float)]


class Marcher(C.Structure):
    _fields_ = [("max_steps", C.c_uint32), ("max_dist", C.c_float), ("eps", C.c_float), ("step_scale", C.c_float),
                ("shadow_steps", C.c_uint32), ("ao_samples", C.c_uint32), ("lod_footprint", C.c_float),
                ("subitize", C.c_float), ("secant", C.c_uint32), ("normal_h", C.c_float)]


class Post(C.Structure):
    _fields_ = [("exposure", C.c_float), ("bloom", C.c_uint32), ("bloom_threshold", C.c_float),
                ("bloom_intensity", C.c_float), ("bloom_radius", C.c_uint32)]


class CsgNode(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("a", C.c_uint32), ("b", C.c_uint32), ("pad", C.c_uint32),
                ("params", C.c_float * 7), ("rot", C.c_float * 9), ("pos", F3), ("scale", C.c_float)]


class Volume(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("min", F3), ("cell", F3),
                ("data", C.POINTER(C.c_float))]


class Gi(C.Structure):
    _fields_ = [("min", F3), ("size", F3), ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
                ("cubes", C.POINTER(C.c_float))]


class SceneDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32),
                ("objects", C.POINTER(Object)), ("n_objects", C.c_uint32),
                ("materials", C.POINTER(Material)), ("n_materials", C.c_uint32),
                ("lights", C.POINTER(Light)), ("n_lights", C.c_uint32),
                ("sun_dir", F3), ("ambient", F3), ("sky_ambient", F3), ("fog", F3), ("fog_density", C.c_float),
                ("aa", C.c_uint32), ("bounces", C.c_uint32), ("shadows", C.c_uint32), ("ao", C.c_uint32),
                ("marcher", Marcher), ("post", Post), ("mode", C.c_uint32),
                ("gi", C.POINTER(Gi)),
                ("volumes", C.POINTER(Volume)), ("n_volumes", C.c_uint32),
                ("csg_nodes", C.POINTER(CsgNode)), ("n_csg_nodes", C.c_uint32),
                ("csg_roots", C.POINTER(C.c_uint32)), ("n_csgs", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("eye", F3), ("forward", F3), ("right", F3), ("up", F3), ("fov_scale", C.c_float)]

    def as_dict(self):
        return {k: (list(getattr(self, k)) if k != "fov_scale" else self.fov_scale)
                for k in ("eye", "forward", "right", "up", "fov_scale")}


class DynSphere(C.Structure):
    _fields_ = [("pos", F3), ("radius", C.c_float), ("albedo", F3), ("metallic", C.c_float)]


class RenderStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("total_ms", C.c_double), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("kernel_launches", C.c_uint32)]


class Tuning(C.Structure):
    _fields_ = [("block", C.c_uint32), ("tile_wlog", C.c_uint32), ("unroll", C.c_uint32), ("min_blocks", C.c_uint32)]


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 16), ("launches", C.c_uint32), ("ms", C.c_double)]


class Job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32),
                ("format", C.c_uint32), ("device_out", C.c_void_p), ("host_out", C.c_void_p),
                ("out_bytes", C.c_size_t)]


class BatchConfig(C.Structure):
    _fields_ = [("max_samples", C.c_uint64), ("use_graphs", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("total_ms", C.c_double), ("sequences", C.c_uint32),
                ("kernel_launches", C.c_uint32), ("graph_launches", C.c_uint32), ("samples", C.c_uint64),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64)]


class Mesh(C.Structure):
    _fields_ = [("positions", C.POINTER(C.c_float)), ("n_positions", C.c_uint32),
                ("triangles", C.POINTER(C.c_uint32)), ("n_triangles", C.c_uint32)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_samples", C.c_uint64), ("max_inflight", C.c_uint32),
                ("use_graphs", C.c_uint32), ("plain", C.c_uint32), ("spec_workers", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("scene_id", C.c_uint32), ("new_scene", C.POINTER(SceneDesc)), ("mesh", C.POINTER(Mesh)),
                ("mesh_volume", C.c_uint32), ("mesh_resolution", C.c_uint32), ("mesh_padding", C.c_float),
                ("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32),
                ("host_out", C.c_void_p), ("out_bytes", C.c_size_t)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("scene_id", C.c_uint32), ("submit_ms", C.c_double), ("start_ms", C.c_double),
                ("done_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "completed", "failed", "sequences", "frames_in_sequences",
                                          "scenes_compiled", "scenes_evicted", "mesh_bakes", "mesh_bake_hits",
                                          "admitted_bytes", "peak_admitted_bytes", "budget_bytes",
                                          "reserved_bytes", "scenes_specialized", "spec_pending", "spec_frames")]


class TuneEntry(C.Structure):
    _fields_ = [("tuning", Tuning), ("device_ms", C.c_double)]


# Every symbol include/mm3e_cuda.h declares (checked by the CPU test suite).
EXPORTED_SYMBOLS = [
    "mm3e_abi_version", "mm3e_camera_look_at", "mm3e_orbit_camera", "mm3e_mat3_from_euler", "mm3e_quat_to_mat3",
    "mm3e_light_directional", "mm3e_scene_validate", "mm3e_scene_tape_bytes",
    "mm3e_ctx_create", "mm3e_ctx_destroy", "mm3e_last_error", "mm3e_ctx_sync", "mm3e_ctx_set_stream", "mm3e_ctx_device_info",
    "mm3e_scene_compile", "mm3e_scene_destroy", "mm3e_render", "mm3e_render_linear", "mm3e_render_device",
    "mm3e_bake_gi", "mm3e_scene_get_gi", "mm3e_render_hits", "mm3e_march_rays", "mm3e_field",
    "mm3e_march_rays_noalloc",
    "mm3e_ctx_set_tuning", "mm3e_ctx_get_tuning", "mm3e_ctx_set_profiling", "mm3e_ctx_kernel_times",
    "mm3e_scene_device_bytes", "mm3e_batch_configure", "mm3e_render_batch", "mm3e_autotune",
    "mm3e_scene_parse_mm3e", "mm3e_parsed_scene_desc", "mm3e_parsed_scene_camera", "mm3e_parsed_scene_free",
    "mm3e_scene_write_mm3e", "mm3e_ctx_set_host_writes", "mm3e_ctx_set_tape_wait", "mm3e_scene_autotune", "mm3e_volume_parse_sdfv", "mm3e_volume_write_sdfv",
    "mm3e_bake_mesh_sdf", "mm3e_render_film", "mm3e_render_gbuffer", "mm3e_reproject", "mm3e_scene_specialize", "mm3e_scene_is_specialized", "mm3e_scene_spec_source", "mm3e_spec_compile_check", "mm3e_scene_tape",
    "mm3e_server_create", "mm3e_server_add_scene", "mm3e_server_submit", "mm3e_server_wait", "mm3e_server_get_stats",
    "mm3e_server_replay", "mm3e_server_destroy",
]
