//! Raw declarations of the libmm3e_cuda C ABI (include/mm3e_cuda.h), field for field. Every
//! struct is `#[repr(C)]` with the header's member order and types; `abi_layout_matches` in the
//! tests checks the sizes the header's C layout gives them.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const MM3E_ABI_VERSION: c_int = 2;

pub const MM3E_OK: c_int = 0;
pub const MM3E_ERR_INVALID: c_int = -1;
pub const MM3E_ERR_UNSUPPORTED: c_int = -2;
pub const MM3E_ERR_CUDA: c_int = -3;
pub const MM3E_ERR_NO_MEMORY: c_int = -4;
pub const MM3E_ERR_TIMEOUT: c_int = -6;

pub const MM3E_PRIM_SPHERE: u32 = 0;
pub const MM3E_PRIM_BOX: u32 = 1;
pub const MM3E_PRIM_ROUND_BOX: u32 = 2;
pub const MM3E_PRIM_TORUS: u32 = 3;
pub const MM3E_PRIM_CYLINDER: u32 = 4;
pub const MM3E_PRIM_CAPSULE: u32 = 5;
pub const MM3E_PRIM_CONE: u32 = 6;
pub const MM3E_PRIM_ELLIPSOID: u32 = 7;
pub const MM3E_PRIM_OCTAHEDRON: u32 = 8;
pub const MM3E_PRIM_HEX_PRISM: u32 = 9;
pub const MM3E_PRIM_PLANE: u32 = 10;
pub const MM3E_PRIM_CSG: u32 = 11;
pub const MM3E_PRIM_VOLUME: u32 = 12;
pub const MM3E_PRIM_SURFACE: u32 = 13;

pub const MM3E_COMBINE_UNION: u32 = 0;
pub const MM3E_COMBINE_SMOOTH: u32 = 1;
pub const MM3E_COMBINE_SUBTRACT: u32 = 2;

pub const MM3E_MODE_BEAUTY: u32 = 0;
pub const MM3E_MODE_NORMAL: u32 = 1;
pub const MM3E_MODE_DEPTH: u32 = 2;
pub const MM3E_MODE_AO: u32 = 3;
pub const MM3E_MODE_STEPS: u32 = 4;
pub const MM3E_MODE_ALBEDO: u32 = 5;

pub const MM3E_FB_RGBA_F32: u32 = 0;
pub const MM3E_FB_RGBA8: u32 = 1;

pub const MM3E_CSG_TRANSFORM: u32 = 100;
pub const MM3E_CSG_UNION: u32 = 101;
pub const MM3E_CSG_INTERSECT: u32 = 102;
pub const MM3E_CSG_SUBTRACT: u32 = 103;
pub const MM3E_CSG_SMOOTH_UNION: u32 = 104;
pub const MM3E_CSG_OFFSET: u32 = 105;
pub const MM3E_CSG_SHELL: u32 = 106;

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_object {
    pub prim: u32,
    pub id: u32,
    pub mat: u32,
    pub combine: u32,
    pub smooth_k: f32,
    pub params: [f32; 7],
    pub rot: [f32; 9],
    pub pos: [f32; 3],
    pub scale: f32,
    pub mirror: u32,
    pub repeat: [f32; 3],
    pub twist: f32,
    pub bend: f32,
    pub elongate: [f32; 3],
    pub round: f32,
    pub onion: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_material {
    pub albedo: [f32; 3],
    pub metallic: f32,
    pub specular: f32,
    pub roughness: f32,
    pub reflectivity: f32,
    pub emissive: [f32; 3],
    pub checker: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_light {
    pub vec: [f32; 3],
    pub color: [f32; 3],
    pub directional: u32,
    pub radius: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_marcher {
    pub max_steps: u32,
    pub max_dist: f32,
    pub eps: f32,
    pub step_scale: f32,
    pub shadow_steps: u32,
    pub ao_samples: u32,
    pub lod_footprint: f32,
    pub subitize: f32,
    pub secant: u32,
    pub normal_h: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_post {
    pub exposure: f32,
    pub bloom: u32,
    pub bloom_threshold: f32,
    pub bloom_intensity: f32,
    pub bloom_radius: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_csg_node {
    pub kind: u32,
    pub a: u32,
    pub b: u32,
    pub pad: u32,
    pub params: [f32; 7],
    pub rot: [f32; 9],
    pub pos: [f32; 3],
    pub scale: f32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct mm3e_volume {
    pub nx: u32,
    pub ny: u32,
    pub nz: u32,
    pub min: [f32; 3],
    pub cell: [f32; 3],
    pub data: *const f32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct mm3e_gi {
    pub min: [f32; 3],
    pub size: [f32; 3],
    pub nx: u32,
    pub ny: u32,
    pub nz: u32,
    pub cubes: *const f32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct mm3e_scene_desc {
    pub width: u32,
    pub height: u32,
    pub objects: *const mm3e_object,
    pub n_objects: u32,
    pub materials: *const mm3e_material,
    pub n_materials: u32,
    pub lights: *const mm3e_light,
    pub n_lights: u32,
    pub sun_dir: [f32; 3],
    pub ambient: [f32; 3],
    pub sky_ambient: [f32; 3],
    pub fog: [f32; 3],
    pub fog_density: f32,
    pub aa: u32,
    pub bounces: u32,
    pub shadows: u32,
    pub ao: u32,
    pub marcher: mm3e_marcher,
    pub post: mm3e_post,
    pub mode: u32,
    pub gi: *const mm3e_gi,
    pub volumes: *const mm3e_volume,
    pub n_volumes: u32,
    pub csg_nodes: *const mm3e_csg_node,
    pub n_csg_nodes: u32,
    pub csg_roots: *const u32,
    pub n_csgs: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_camera {
    pub eye: [f32; 3],
    pub forward: [f32; 3],
    pub right: [f32; 3],
    pub up: [f32; 3],
    pub fov_scale: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_dyn_sphere {
    pub pos: [f32; 3],
    pub radius: f32,
    pub albedo: [f32; 3],
    pub metallic: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Default)]
pub struct mm3e_render_stats {
    pub device_ms: f64,
    pub total_ms: f64,
    pub h2d_bytes: u64,
    pub d2h_bytes: u64,
    pub kernel_launches: u32,
}

/// Opaque handles.
#[repr(C)]
pub struct mm3e_ctx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct mm3e_scene {
    _private: [u8; 0],
}

extern "C" {
    pub fn mm3e_abi_version() -> c_int;
    pub fn mm3e_scene_validate(desc: *const mm3e_scene_desc, err: *mut c_char, err_len: usize) -> c_int;
    pub fn mm3e_ctx_create(device: c_int, out: *mut *mut mm3e_ctx) -> c_int;
    pub fn mm3e_ctx_destroy(ctx: *mut mm3e_ctx);
    pub fn mm3e_last_error(ctx: *const mm3e_ctx) -> *const c_char;
    pub fn mm3e_ctx_sync(ctx: *mut mm3e_ctx) -> c_int;
    pub fn mm3e_scene_compile(ctx: *mut mm3e_ctx, desc: *const mm3e_scene_desc, out: *mut *mut mm3e_scene) -> c_int;
    pub fn mm3e_scene_destroy(scene: *mut mm3e_scene);
    pub fn mm3e_scene_specialize(scene: *mut mm3e_scene, mode: c_int, compile_ms: *mut f64) -> c_int;
    pub fn mm3e_render(
        scene: *mut mm3e_scene,
        camera: *const mm3e_camera,
        dyn_spheres: *const mm3e_dyn_sphere,
        n_dyn: usize,
        format: u32,
        host_out: *mut c_void,
        out_bytes: usize,
        stats: *mut mm3e_render_stats,
    ) -> c_int;
    pub fn mm3e_render_linear(
        scene: *mut mm3e_scene,
        camera: *const mm3e_camera,
        host_rgb: *mut f32,
        n_floats: usize,
    ) -> c_int;
    pub fn mm3e_bake_gi(scene: *mut mm3e_scene, nx: u32, ny: u32, nz: u32, samples: u32) -> c_int;
}
