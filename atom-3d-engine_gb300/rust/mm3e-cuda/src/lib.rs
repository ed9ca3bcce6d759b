//! mm3e-cuda — MM3E's per-pixel SDF render path on an NVIDIA GB300 (sm_103a), behind the same
//! calls as the CPU backend.
//!
//! The shape mirrors `mm3e_cpu_parallel` (mm3e-cpu-parallel/src/lib.rs:26-118): a renderer
//! compiles an `Arc<Scene>` once into a device-resident scene, and the compiled scene renders a
//! camera (plus dynamic spheres) into the `Framebuffer` that `render_with_threads_checked`
//! (mm3e-orchestrator/src/lib.rs:866-871) returns for the same inputs: straight-alpha RGBA f32,
//! alpha 1, post-processed. Errors are the `Err(String)` of the checked reference calls, with the
//! library's message (mm3e_last_error).
//!
//! ```ignore
//! let renderer = CudaRenderer::new(0)?;                       // device 0
//! let compiled = renderer.compile(Arc::new(scene))?;           // validate + lower once
//! let fb: Framebuffer = compiled.try_render(&camera, &[])?;    // per camera
//! ```
//!
//! The marshalling below (`SceneDesc::new`) turns `&Scene` into the flat `mm3e_scene_desc` of
//! include/mm3e_cuda.h: objects with their primitive parameters packed as the header documents,
//! materials, lights, marcher, post, render mode, GI probes, SDF volumes and the CSG
//! expressions as one node array (children before parents) with a root per expression.
//! UV appearance bindings and native triangle surfaces are refused, as the reference's GPU twin
//! refuses them (mm3e-gpu/src/wgsl.rs:41-47).

pub mod ffi;

use std::ffi::CStr;
use std::ptr;
use std::sync::{Arc, Mutex};

use mm3e_cpu_parallel::DynSphere;
use mm3e_kit::camera::Camera;
use mm3e_kit::color::Rgba;
use mm3e_kit::csg::Expr;
use mm3e_kit::framebuffer::Framebuffer;
use mm3e_kit::vec::{Transform, Vec3};
use mm3e_orchestrator::{Combine, Prim, RenderMode, Scene};

fn v3(v: Vec3) -> [f32; 3] {
    [v.x, v.y, v.z]
}

fn rot9(t: &Transform) -> [f32; 9] {
    let c = &t.rot.cols;
    [c[0].x, c[0].y, c[0].z, c[1].x, c[1].y, c[1].z, c[2].x, c[2].y, c[2].z]
}

/// Primitive kind and its 7 parameters as the header packs them (include/mm3e_cuda.h, Prim).
fn prim_params(p: &Prim) -> Result<(u32, u32, [f32; 7]), String> {
    let mut q = [0.0f32; 7];
    let (kind, id) = match *p {
        Prim::Sphere { r } => {
            q[0] = r;
            (ffi::MM3E_PRIM_SPHERE, 0)
        }
        Prim::Box { half } => {
            q[..3].copy_from_slice(&v3(half));
            (ffi::MM3E_PRIM_BOX, 0)
        }
        Prim::RoundBox { half, radius } => {
            q[..3].copy_from_slice(&v3(half));
            q[3] = radius;
            (ffi::MM3E_PRIM_ROUND_BOX, 0)
        }
        Prim::Torus { major, minor } => {
            q[0] = major;
            q[1] = minor;
            (ffi::MM3E_PRIM_TORUS, 0)
        }
        Prim::Cylinder { h, r } => {
            q[0] = h;
            q[1] = r;
            (ffi::MM3E_PRIM_CYLINDER, 0)
        }
        Prim::Capsule { a, b, r } => {
            q[..3].copy_from_slice(&v3(a));
            q[3..6].copy_from_slice(&v3(b));
            q[6] = r;
            (ffi::MM3E_PRIM_CAPSULE, 0)
        }
        Prim::Cone { r1, r2, h } => {
            q[0] = r1;
            q[1] = r2;
            q[2] = h;
            (ffi::MM3E_PRIM_CONE, 0)
        }
        Prim::Ellipsoid { r } => {
            q[..3].copy_from_slice(&v3(r));
            (ffi::MM3E_PRIM_ELLIPSOID, 0)
        }
        Prim::Octahedron { s } => {
            q[0] = s;
            (ffi::MM3E_PRIM_OCTAHEDRON, 0)
        }
        Prim::HexPrism { r, h } => {
            q[0] = r;
            q[1] = h;
            (ffi::MM3E_PRIM_HEX_PRISM, 0)
        }
        Prim::Plane { n, h } => {
            q[..3].copy_from_slice(&v3(n));
            q[3] = h;
            (ffi::MM3E_PRIM_PLANE, 0)
        }
        Prim::Csg { id } => (ffi::MM3E_PRIM_CSG, id),
        Prim::Volume { id } => (ffi::MM3E_PRIM_VOLUME, id),
        Prim::Surface { .. } => {
            return Err("native triangle surfaces are not supported by the GPU backend; use the CPU renderer".into())
        }
    };
    Ok((kind, id, q))
}

/// One csg::Expr tree appended to `nodes`, children first; returns the root's index
/// (mm3e-kit/src/csg.rs:17-92; the header's mm3e_csg_node).
fn flatten_expr(e: &Expr, nodes: &mut Vec<ffi::mm3e_csg_node>) -> u32 {
    let mut n = ffi::mm3e_csg_node { scale: 1.0, ..Default::default() };
    n.rot = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0];
    match e {
        Expr::Sphere { r } => {
            n.kind = ffi::MM3E_PRIM_SPHERE;
            n.params[0] = *r;
        }
        Expr::Box { half } => {
            n.kind = ffi::MM3E_PRIM_BOX;
            n.params[..3].copy_from_slice(&v3(*half));
        }
        Expr::RoundBox { half, radius } => {
            n.kind = ffi::MM3E_PRIM_ROUND_BOX;
            n.params[..3].copy_from_slice(&v3(*half));
            n.params[3] = *radius;
        }
        Expr::Torus { major, minor } => {
            n.kind = ffi::MM3E_PRIM_TORUS;
            n.params[0] = *major;
            n.params[1] = *minor;
        }
        Expr::Cylinder { h, r } => {
            n.kind = ffi::MM3E_PRIM_CYLINDER;
            n.params[0] = *h;
            n.params[1] = *r;
        }
        Expr::Capsule { a, b, r } => {
            n.kind = ffi::MM3E_PRIM_CAPSULE;
            n.params[..3].copy_from_slice(&v3(*a));
            n.params[3..6].copy_from_slice(&v3(*b));
            n.params[6] = *r;
        }
        Expr::Cone { r1, r2, h } => {
            n.kind = ffi::MM3E_PRIM_CONE;
            n.params[0] = *r1;
            n.params[1] = *r2;
            n.params[2] = *h;
        }
        Expr::Ellipsoid { r } => {
            n.kind = ffi::MM3E_PRIM_ELLIPSOID;
            n.params[..3].copy_from_slice(&v3(*r));
        }
        Expr::Octahedron { s } => {
            n.kind = ffi::MM3E_PRIM_OCTAHEDRON;
            n.params[0] = *s;
        }
        Expr::HexPrism { r, h } => {
            n.kind = ffi::MM3E_PRIM_HEX_PRISM;
            n.params[0] = *r;
            n.params[1] = *h;
        }
        Expr::Plane { n: nv, h } => {
            n.kind = ffi::MM3E_PRIM_PLANE;
            n.params[..3].copy_from_slice(&v3(*nv));
            n.params[3] = *h;
        }
        Expr::Transform { shape, xform } => {
            n.kind = ffi::MM3E_CSG_TRANSFORM;
            n.a = flatten_expr(shape, nodes);
            n.rot = rot9(xform);
            n.pos = v3(xform.pos);
            n.scale = xform.scale;
        }
        Expr::Union { a, b } => {
            n.kind = ffi::MM3E_CSG_UNION;
            n.a = flatten_expr(a, nodes);
            n.b = flatten_expr(b, nodes);
        }
        Expr::Intersect { a, b } => {
            n.kind = ffi::MM3E_CSG_INTERSECT;
            n.a = flatten_expr(a, nodes);
            n.b = flatten_expr(b, nodes);
        }
        Expr::Subtract { a, b } => {
            n.kind = ffi::MM3E_CSG_SUBTRACT;
            n.a = flatten_expr(a, nodes);
            n.b = flatten_expr(b, nodes);
        }
        Expr::SmoothUnion { a, b, k } => {
            n.kind = ffi::MM3E_CSG_SMOOTH_UNION;
            n.params[0] = *k;
            n.a = flatten_expr(a, nodes);
            n.b = flatten_expr(b, nodes);
        }
        Expr::Offset { shape, distance } => {
            n.kind = ffi::MM3E_CSG_OFFSET;
            n.params[0] = *distance;
            n.a = flatten_expr(shape, nodes);
        }
        Expr::Shell { shape, thickness } => {
            n.kind = ffi::MM3E_CSG_SHELL;
            n.params[0] = *thickness;
            n.a = flatten_expr(shape, nodes);
        }
    }
    nodes.push(n);
    (nodes.len() - 1) as u32
}

fn mode_code(m: RenderMode) -> u32 {
    match m {
        RenderMode::Beauty => ffi::MM3E_MODE_BEAUTY,
        RenderMode::Normal => ffi::MM3E_MODE_NORMAL,
        RenderMode::Depth => ffi::MM3E_MODE_DEPTH,
        RenderMode::Ao => ffi::MM3E_MODE_AO,
        RenderMode::Steps => ffi::MM3E_MODE_STEPS,
        RenderMode::Albedo => ffi::MM3E_MODE_ALBEDO,
    }
}

fn count(n: usize, what: &str) -> Result<u32, String> {
    u32::try_from(n).map_err(|_| format!("too many {what} for the GPU backend"))
}

/// A `&Scene` marshalled into `mm3e_scene_desc`, with the arrays it points into. The C ABI copies
/// what it keeps during mm3e_scene_compile, so this lives only for that call.
pub struct SceneDesc {
    desc: ffi::mm3e_scene_desc,
    _objects: Vec<ffi::mm3e_object>,
    _materials: Vec<ffi::mm3e_material>,
    _lights: Vec<ffi::mm3e_light>,
    _volumes: Vec<ffi::mm3e_volume>,
    _csg_nodes: Vec<ffi::mm3e_csg_node>,
    _csg_roots: Vec<u32>,
    _gi: Option<Box<ffi::mm3e_gi>>,
    _gi_cubes: Vec<f32>,
}

impl SceneDesc {
    /// Scene (mm3e-orchestrator/src/lib.rs:561-592) field by field.
    pub fn new(scene: &Scene) -> Result<SceneDesc, String> {
        if !scene.appearance.is_empty() {
            return Err("UV surface textures are not supported by the GPU backend; use the CPU renderer".into());
        }
        if !scene.surfaces.is_empty() {
            return Err("native triangle surfaces are not supported by the GPU backend; use the CPU renderer".into());
        }
        let mut objects = Vec::with_capacity(scene.objects.len());
        for o in &scene.objects {
            let (prim, id, params) = prim_params(&o.prim)?;
            let m = &o.mods;
            let (combine, smooth_k) = match o.combine {
                Combine::Union => (ffi::MM3E_COMBINE_UNION, 0.0),
                Combine::Smooth(k) => (ffi::MM3E_COMBINE_SMOOTH, k),
                Combine::Subtract => (ffi::MM3E_COMBINE_SUBTRACT, 0.0),
            };
            objects.push(ffi::mm3e_object {
                prim,
                id,
                mat: o.mat,
                combine,
                smooth_k,
                params,
                rot: rot9(&o.xform),
                pos: v3(o.xform.pos),
                scale: o.xform.scale,
                mirror: (m.mirror[0] as u32) | (m.mirror[1] as u32) << 1 | (m.mirror[2] as u32) << 2,
                repeat: v3(m.repeat),
                twist: m.twist,
                bend: m.bend,
                elongate: v3(m.elongate),
                round: m.round,
                onion: m.onion,
            });
        }
        let materials: Vec<ffi::mm3e_material> = scene
            .materials
            .iter()
            .map(|m| ffi::mm3e_material {
                albedo: v3(m.albedo),
                metallic: m.metallic,
                specular: m.specular,
                roughness: m.roughness,
                reflectivity: m.reflectivity,
                emissive: v3(m.emissive),
                checker: m.checker as u32,
            })
            .collect();
        let lights: Vec<ffi::mm3e_light> = scene
            .lights
            .iter()
            .map(|l| ffi::mm3e_light {
                vec: v3(l.vec),
                color: v3(l.color),
                directional: l.directional as u32,
                radius: l.radius,
            })
            .collect();
        let volumes: Vec<ffi::mm3e_volume> = scene
            .volumes
            .iter()
            .map(|v| {
                let (nx, ny, nz) = v.dims;
                Ok(ffi::mm3e_volume {
                    nx: count(nx, "volume samples")?,
                    ny: count(ny, "volume samples")?,
                    nz: count(nz, "volume samples")?,
                    min: v3(v.min),
                    cell: v3(v.cell),
                    data: v.data.as_ptr(),
                })
            })
            .collect::<Result<_, String>>()?;
        let mut csg_nodes = Vec::new();
        let csg_roots: Vec<u32> = scene.csgs.iter().map(|e| flatten_expr(e, &mut csg_nodes)).collect();
        // GiVolume::raw (gi.rs:133-135): cubes of 6 faces x rgb per probe, probes (k*ny + j)*nx + i
        let mut gi_cubes = Vec::new();
        let gi = match &scene.gi {
            None => None,
            Some(g) => {
                let (min, size, (nx, ny, nz), cubes) = g.raw();
                gi_cubes.reserve(cubes.len() * 18);
                for probe in cubes {
                    for face in probe {
                        gi_cubes.extend_from_slice(&v3(*face));
                    }
                }
                Some(Box::new(ffi::mm3e_gi {
                    min: v3(min),
                    size: v3(size),
                    nx: count(nx, "GI probes")?,
                    ny: count(ny, "GI probes")?,
                    nz: count(nz, "GI probes")?,
                    cubes: gi_cubes.as_ptr(),
                }))
            }
        };
        let mk = &scene.marcher;
        let pp = &scene.post;
        let desc = ffi::mm3e_scene_desc {
            width: scene.width,
            height: scene.height,
            objects: objects.as_ptr(),
            n_objects: count(objects.len(), "objects")?,
            materials: materials.as_ptr(),
            n_materials: count(materials.len(), "materials")?,
            lights: lights.as_ptr(),
            n_lights: count(lights.len(), "lights")?,
            sun_dir: v3(scene.sun_dir),
            ambient: v3(scene.ambient),
            sky_ambient: v3(scene.sky_ambient),
            fog: v3(scene.fog),
            fog_density: scene.fog_density,
            aa: scene.aa,
            bounces: scene.bounces,
            shadows: scene.shadows as u32,
            ao: scene.ao as u32,
            marcher: ffi::mm3e_marcher {
                max_steps: mk.max_steps,
                max_dist: mk.max_dist,
                eps: mk.eps,
                step_scale: mk.step_scale,
                shadow_steps: mk.shadow_steps,
                ao_samples: mk.ao_samples,
                lod_footprint: mk.lod_footprint,
                subitize: mk.subitize,
                secant: mk.secant as u32,
                normal_h: mk.normal_h,
            },
            post: ffi::mm3e_post {
                exposure: pp.exposure,
                bloom: pp.bloom as u32,
                bloom_threshold: pp.bloom_threshold,
                bloom_intensity: pp.bloom_intensity,
                bloom_radius: pp.bloom_radius,
            },
            mode: mode_code(scene.mode),
            gi: gi.as_deref().map_or(ptr::null(), |g| g as *const ffi::mm3e_gi),
            volumes: if volumes.is_empty() { ptr::null() } else { volumes.as_ptr() },
            n_volumes: count(volumes.len(), "volumes")?,
            csg_nodes: if csg_nodes.is_empty() { ptr::null() } else { csg_nodes.as_ptr() },
            n_csg_nodes: count(csg_nodes.len(), "CSG nodes")?,
            csg_roots: if csg_roots.is_empty() { ptr::null() } else { csg_roots.as_ptr() },
            n_csgs: count(csg_roots.len(), "CSG expressions")?,
        };
        Ok(SceneDesc {
            desc,
            _objects: objects,
            _materials: materials,
            _lights: lights,
            _volumes: volumes,
            _csg_nodes: csg_nodes,
            _csg_roots: csg_roots,
            _gi: gi,
            _gi_cubes: gi_cubes,
        })
    }

    pub fn as_ffi(&self) -> *const ffi::mm3e_scene_desc {
        &self.desc
    }
}

fn camera_ffi(c: &Camera) -> ffi::mm3e_camera {
    ffi::mm3e_camera { eye: v3(c.eye), forward: v3(c.forward), right: v3(c.right), up: v3(c.up), fov_scale: c.fov_scale }
}

/// One device context (mm3e_ctx). The C ABI's contexts are not thread-safe, so every call takes
/// this mutex; compiled scenes share their renderer's context.
struct Context {
    ctx: Mutex<*mut ffi::mm3e_ctx>,
}

// The raw context is only used under the mutex.
unsafe impl Send for Context {}
unsafe impl Sync for Context {}

impl Context {
    fn error(ctx: *mut ffi::mm3e_ctx, rc: i32, what: &str) -> String {
        let msg = unsafe { CStr::from_ptr(ffi::mm3e_last_error(ctx)) }.to_string_lossy().into_owned();
        if msg.is_empty() {
            format!("{what} failed (code {rc})")
        } else {
            msg
        }
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        let ctx = *self.ctx.lock().unwrap_or_else(|e| e.into_inner());
        if !ctx.is_null() {
            unsafe { ffi::mm3e_ctx_destroy(ctx) };
        }
    }
}

/// The GPU counterpart of `CpuParallelRenderer` (mm3e-cpu-parallel/src/lib.rs:86-112).
pub struct CudaRenderer {
    ctx: Arc<Context>,
    specialize: bool,
}

impl CudaRenderer {
    /// A renderer on CUDA device `device`.
    pub fn new(device: i32) -> Result<Self, String> {
        if unsafe { ffi::mm3e_abi_version() } != ffi::MM3E_ABI_VERSION {
            return Err("libmm3e_cuda ABI version does not match this crate".into());
        }
        let mut ctx = ptr::null_mut();
        let rc = unsafe { ffi::mm3e_ctx_create(device, &mut ctx) };
        if rc != ffi::MM3E_OK {
            return Err(format!("no CUDA context on device {device} (code {rc})"));
        }
        Ok(Self { ctx: Arc::new(Context { ctx: Mutex::new(ctx) }), specialize: true })
    }

    /// Whether compiled fixed scenes get scene-specialised march / shadow / AO kernels (NVRTC,
    /// on by default for fields of up to 64 objects). Frames are identical either way.
    pub fn with_specialization(mut self, on: bool) -> Self {
        self.specialize = on;
        self
    }

    /// Validate and lower `scene` into a device-resident scene (CpuParallelRenderer::compile,
    /// GpuRenderer::compile_checked). The source is retained and never modified.
    pub fn compile(&self, scene: Arc<Scene>) -> Result<CudaScene, String> {
        let desc = SceneDesc::new(&scene)?;
        let ctx = self.ctx.ctx.lock().map_err(|_| "CUDA context poisoned".to_string())?;
        let mut handle = ptr::null_mut();
        let rc = unsafe { ffi::mm3e_scene_compile(*ctx, desc.as_ffi(), &mut handle) };
        if rc != ffi::MM3E_OK {
            return Err(Context::error(*ctx, rc, "mm3e_scene_compile"));
        }
        if self.specialize {
            let mut ms = 0.0f64;
            let rc = unsafe { ffi::mm3e_scene_specialize(handle, 1, &mut ms) };
            if rc != ffi::MM3E_OK {
                // the tape interpreter renders the same frames: keep it and report nothing
                let _ = Context::error(*ctx, rc, "mm3e_scene_specialize");
            }
        }
        drop(ctx);
        Ok(CudaScene { ctx: Arc::clone(&self.ctx), scene: handle, source: scene })
    }
}

/// A compiled scene: the GPU counterpart of `CpuParallelScene` (mm3e-cpu-parallel/src/lib.rs:26-66).
pub struct CudaScene {
    ctx: Arc<Context>,
    scene: *mut ffi::mm3e_scene,
    source: Arc<Scene>,
}

// The raw scene handle is only used under the context's mutex.
unsafe impl Send for CudaScene {}
unsafe impl Sync for CudaScene {}

impl Drop for CudaScene {
    fn drop(&mut self) {
        let _guard = self.ctx.ctx.lock().unwrap_or_else(|e| e.into_inner());
        unsafe { ffi::mm3e_scene_destroy(self.scene) };
    }
}

impl CudaScene {
    /// The retained source scene.
    pub fn scene(&self) -> &Arc<Scene> {
        &self.source
    }

    /// Render through the GPU path. Invalid dynamic input panics with a validation message, as
    /// CpuParallelScene::render does; use [`Self::try_render`] for external data.
    pub fn render(&self, camera: &Camera, dyn_spheres: &[DynSphere]) -> Framebuffer {
        self.try_render(camera, dyn_spheres).expect("invalid dynamic sphere render input")
    }

    /// CpuParallelScene::try_render: dynamic spheres are validated (finite position, positive
    /// radius, albedo / metallic in [0,1]) and rendered as real objects with default materials;
    /// the source is never modified. Returns the post-processed RGBA f32 framebuffer.
    pub fn try_render(&self, camera: &Camera, dyn_spheres: &[DynSphere]) -> Result<Framebuffer, String> {
        let (w, h) = (self.source.width, self.source.height);
        let n = (w as usize).checked_mul(h as usize).ok_or("framebuffer dimensions overflow addressable memory")?;
        let mut rgba = vec![0.0f32; n * 4];
        let dyn_ffi: Vec<ffi::mm3e_dyn_sphere> = dyn_spheres
            .iter()
            .map(|s| ffi::mm3e_dyn_sphere { pos: v3(s.pos), radius: s.radius, albedo: v3(s.albedo), metallic: s.metallic })
            .collect();
        let cam = camera_ffi(camera);
        {
            let ctx = self.ctx.ctx.lock().map_err(|_| "CUDA context poisoned".to_string())?;
            let rc = unsafe {
                ffi::mm3e_render(
                    self.scene,
                    &cam,
                    if dyn_ffi.is_empty() { ptr::null() } else { dyn_ffi.as_ptr() },
                    dyn_ffi.len(),
                    ffi::MM3E_FB_RGBA_F32,
                    rgba.as_mut_ptr() as *mut std::os::raw::c_void,
                    rgba.len() * std::mem::size_of::<f32>(),
                    ptr::null_mut(),
                )
            };
            if rc != ffi::MM3E_OK {
                return Err(Context::error(*ctx, rc, "mm3e_render"));
            }
        }
        let mut fb = Framebuffer::new(w, h, Rgba::new(0.0, 0.0, 0.0, 0.0));
        for y in 0..h {
            for x in 0..w {
                let i = (y as usize * w as usize + x as usize) * 4;
                fb.put(x, y, Rgba::new(rgba[i], rgba[i + 1], rgba[i + 2], rgba[i + 3]));
            }
        }
        Ok(fb)
    }

    /// The frame as RGBA8 bytes (`Framebuffer::to_rgba8` over black), the GPU twin's
    /// GpuScene::render_rgba_dyn output shape (mm3e-gpu/src/lib.rs:377-402).
    pub fn render_rgba(&self, camera: &Camera, dyn_spheres: &[DynSphere]) -> Result<Vec<u8>, String> {
        let (w, h) = (self.source.width as usize, self.source.height as usize);
        let mut out = vec![0u8; w.checked_mul(h).and_then(|n| n.checked_mul(4)).ok_or("framebuffer too large")?];
        let dyn_ffi: Vec<ffi::mm3e_dyn_sphere> = dyn_spheres
            .iter()
            .map(|s| ffi::mm3e_dyn_sphere { pos: v3(s.pos), radius: s.radius, albedo: v3(s.albedo), metallic: s.metallic })
            .collect();
        let cam = camera_ffi(camera);
        let ctx = self.ctx.ctx.lock().map_err(|_| "CUDA context poisoned".to_string())?;
        let rc = unsafe {
            ffi::mm3e_render(
                self.scene,
                &cam,
                if dyn_ffi.is_empty() { ptr::null() } else { dyn_ffi.as_ptr() },
                dyn_ffi.len(),
                ffi::MM3E_FB_RGBA8,
                out.as_mut_ptr() as *mut std::os::raw::c_void,
                out.len(),
                ptr::null_mut(),
            )
        };
        if rc != ffi::MM3E_OK {
            return Err(Context::error(*ctx, rc, "mm3e_render"));
        }
        Ok(out)
    }

    /// render_linear_with_threads_checked (lib.rs:902-907): beauty radiance before post.
    pub fn render_linear(&self, camera: &Camera) -> Result<Vec<Vec3>, String> {
        let n = self.source.width as usize * self.source.height as usize;
        let mut rgb = vec![0.0f32; n * 3];
        let cam = camera_ffi(camera);
        let ctx = self.ctx.ctx.lock().map_err(|_| "CUDA context poisoned".to_string())?;
        let rc = unsafe { ffi::mm3e_render_linear(self.scene, &cam, rgb.as_mut_ptr(), rgb.len()) };
        if rc != ffi::MM3E_OK {
            return Err(Context::error(*ctx, rc, "mm3e_render_linear"));
        }
        Ok(rgb.chunks_exact(3).map(|c| Vec3::new(c[0], c[1], c[2])).collect())
    }

    /// Scene::bake_gi on the GPU (gi.rs:38-125): replaces this compiled scene's probe volume
    /// (`dims` probes, `samples` rays per probe face); the source scene is unchanged.
    pub fn bake_gi(&self, dims: (u32, u32, u32), samples: u32) -> Result<(), String> {
        let ctx = self.ctx.ctx.lock().map_err(|_| "CUDA context poisoned".to_string())?;
        let rc = unsafe { ffi::mm3e_bake_gi(self.scene, dims.0, dims.1, dims.2, samples) };
        if rc != ffi::MM3E_OK {
            return Err(Context::error(*ctx, rc, "mm3e_bake_gi"));
        }
        Ok(())
    }
}

/// render_with_threads_checked (mm3e-orchestrator/src/lib.rs:866-871) on the GPU: compile
/// `scene` and render one frame. For repeated frames of one scene keep the [`CudaScene`].
pub fn render_checked(renderer: &CudaRenderer, scene: &Scene, camera: &Camera) -> Result<Framebuffer, String> {
    renderer.with_scene_once(scene, |s| s.try_render(camera, &[]))
}

impl CudaRenderer {
    fn with_scene_once<R>(&self, scene: &Scene, f: impl FnOnce(&CudaScene) -> Result<R, String>) -> Result<R, String> {
        let compiled = CudaRenderer { ctx: Arc::clone(&self.ctx), specialize: false }.compile(Arc::new(scene.clone()))?;
        f(&compiled)
    }
}

#[cfg(test)]
mod tests {
    use super::ffi::*;
    use std::mem::size_of;

    #[test]
    fn abi_layout_matches() {
        // the sizes the C compiler gives the header's structs on LP64 hosts
        assert_eq!(size_of::<mm3e_object>(), 4 * 4 + 4 + 7 * 4 + 9 * 4 + 3 * 4 + 4 + 4 + 3 * 4 + 4 + 4 + 3 * 4 + 4 + 4);
        assert_eq!(size_of::<mm3e_material>(), 11 * 4);
        assert_eq!(size_of::<mm3e_light>(), 8 * 4);
        assert_eq!(size_of::<mm3e_camera>(), 13 * 4);
        assert_eq!(size_of::<mm3e_dyn_sphere>(), 8 * 4);
        assert_eq!(size_of::<mm3e_marcher>(), 10 * 4);
        assert_eq!(size_of::<mm3e_post>(), 5 * 4);
        assert_eq!(size_of::<mm3e_csg_node>(), 4 * 4 + 7 * 4 + 9 * 4 + 3 * 4 + 4);
    }
}
