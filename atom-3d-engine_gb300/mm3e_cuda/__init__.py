"""mm3e_cuda — GB300 (sm_103a) drop-in for MM3E's per-pixel SDF render path.

Host-side mirror of the reference's render interface over the C ABI (include/mm3e_cuda.h):

    scene = Scene(960, 540)              # mm3e_orchestrator::Scene
    ...                                  # materials / objects / lights as in the reference
    fb = render(scene, camera)           # mm3e_orchestrator::render -> RGBA f32 (h, w, 4)

    renderer = CudaRenderer()            # CpuParallelRenderer counterpart (mm3e-cpu-parallel)
    compiled = renderer.compile(scene)   # CpuParallelRenderer::compile / GpuRenderer::compile
    fb = compiled.try_render(camera, dyn_spheres)   # CpuParallelScene::try_render

Every call runs on the GPU through libmm3e_cuda.so; there is no CPU fallback. Errors from the
checked reference calls (`Err(String)`) surface as RenderError with the library's message.
"""
import ctypes as C
import weakref

import numpy as np

from . import abi
from .native import NativeLibraryMissing, lib
from .scene import (DynSphere, Expr, GiVolume, Light, Marcher, Material, Object, Post, Prim, Scene, SdfVolume,
                    Transform, directional, look_at, mat3_from_euler, normalize_f32, orbit_camera, quat_to_mat3,
                    radians)

RenderMode = abi  # RenderMode.MODE_* constants


class RenderError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{message} (code {code})")
        self.code = code
        self.message = message


class Context:
    """One CUDA stream on one device (mm3e_ctx)."""

    def __init__(self, device=0):
        self._ptr = C.c_void_p()
        self._scenes = weakref.WeakSet()
        rc = lib().mm3e_ctx_create(device, C.byref(self._ptr))
        if rc != abi.OK:
            raise RenderError(rc, f"mm3e_ctx_create(device={device}) failed")
        self.device = device

    @property
    def handle(self):
        return self._ptr

    def check(self, rc):
        if rc != abi.OK:
            raise RenderError(rc, lib().mm3e_last_error(self._ptr).decode(errors="replace"))

    def sync(self):
        self.check(lib().mm3e_ctx_sync(self._ptr))

    def set_stream(self, cuda_stream_handle):
        """Issue all work on a caller-owned cudaStream_t (an int handle, e.g. torch's
        `stream.cuda_stream`); None restores the context's own stream."""
        self.check(lib().mm3e_ctx_set_stream(self._ptr, C.c_void_p(cuda_stream_handle or 0)))

    def device_info(self):
        sm, clk = C.c_int(), C.c_int()
        self.check(lib().mm3e_ctx_device_info(self._ptr, C.byref(sm), C.byref(clk)))
        return {"sm_count": sm.value, "clock_khz": clk.value}

    # ---- launch shape, profiling -------------------------------------------------------------
    def set_tuning(self, block=128, tile_wlog=3, unroll=64, min_blocks=0):
        self.check(lib().mm3e_ctx_set_tuning(self._ptr, C.byref(abi.Tuning(block, tile_wlog, unroll, min_blocks))))

    def get_tuning(self):
        t = abi.Tuning()
        self.check(lib().mm3e_ctx_get_tuning(self._ptr, C.byref(t)))
        return {"block": t.block, "tile_wlog": t.tile_wlog, "unroll": t.unroll, "min_blocks": t.min_blocks}

    def set_profiling(self, on=True):
        self.check(lib().mm3e_ctx_set_profiling(self._ptr, 1 if on else 0))

    def set_host_writes(self, on=True):
        """Direct kernel writes into host framebuffers where the device shares the host's page
        tables (default on); returns whether they are in use."""
        active = C.c_int()
        self.check(lib().mm3e_ctx_set_host_writes(self._ptr, 1 if on else 0, C.byref(active)))
        return bool(active.value)

    def set_tape_wait(self, limit=0, probe=False):
        """Iteration limit of the kernels' tape-staging wait (0: the default); probe=True issues no
        tape copy so that the wait runs out (renders then fail with ERR_TIMEOUT)."""
        self.check(lib().mm3e_ctx_set_tape_wait(self._ptr, int(limit), 1 if probe else 0))

    def kernel_times(self):
        """{kind: (launches, ms)} of the passes run since the last call (profiling on)."""
        arr = (abi.KernelTime * 16)()
        n = C.c_uint32()
        self.check(lib().mm3e_ctx_kernel_times(self._ptr, arr, 16, C.byref(n)))
        return {arr[i].name.decode(): (arr[i].launches, arr[i].ms) for i in range(min(n.value, 16))}

    # ---- batched rendering ---------------------------------------------------------------------
    def configure_batch(self, max_samples=0, use_graphs=True):
        self.check(lib().mm3e_batch_configure(self._ptr, C.byref(abi.BatchConfig(max_samples, 1 if use_graphs else 0))))

    @staticmethod
    def make_jobs(items):
        """items: (CompiledScene, camera, width, height, format, device_ptr or None, host ndarray or None)."""
        jobs = (abi.Job * len(items))()
        for i, (sc, cam, w, h, fmt, dptr, host) in enumerate(items):
            j = jobs[i]
            j.scene = sc._ptr
            j.camera = cam
            j.width, j.height, j.format = w, h, fmt
            px = 4 if fmt == abi.FB_RGBA8 else 16
            j.out_bytes = (w or sc.width) * (h or sc.height) * px
            if dptr:
                j.device_out = dptr
            else:
                j.host_out = host.ctypes.data
        return jobs

    def render_batch(self, jobs, n=None):
        """Render a ctypes Job array (see make_jobs); returns the batch stats as a dict."""
        st = abi.BatchStats()
        self.check(lib().mm3e_render_batch(self._ptr, jobs, len(jobs) if n is None else n, C.byref(st)))
        return {k: getattr(st, k) for k, _ in abi.BatchStats._fields_}

    def autotune(self, jobs, repeats=1):
        best = abi.Tuning()
        rep = (abi.TuneEntry * 64)()
        n = C.c_uint32()
        self.check(lib().mm3e_autotune(self._ptr, jobs, len(jobs), repeats, C.byref(best), rep, 64, C.byref(n)))
        table = [({"block": rep[i].tuning.block, "tile_wlog": rep[i].tuning.tile_wlog,
                   "unroll": rep[i].tuning.unroll, "min_blocks": rep[i].tuning.min_blocks}, rep[i].device_ms)
                 for i in range(n.value)]
        return {"block": best.block, "tile_wlog": best.tile_wlog, "unroll": best.unroll,
                "min_blocks": best.min_blocks}, table

    # ---- reprojection -------------------------------------------------------------------------------
    def reproject(self, gframe, new_camera, mover_deltas=(), hybrid_scene=None):
        """reproject::reproject (reproject.rs:118), or reproject_hybrid (lib.rs:1040) with
        `hybrid_scene` (a CompiledScene): the G-buffer frame `gframe` (render_gbuffer's dict)
        warped into `new_camera`; (h, w, 4) u8."""
        h, w = gframe["depth"].shape
        color = np.ascontiguousarray(gframe["color"], np.uint8)
        depth = np.ascontiguousarray(gframe["depth"], np.float32)
        obj = np.ascontiguousarray(gframe["obj"], np.int32)
        if color.shape != (h, w, 4) or obj.shape != (h, w):
            raise ValueError("G-buffer frame arrays disagree in shape")
        dl = np.ascontiguousarray(np.asarray(mover_deltas, np.float32).reshape(-1, 3))
        out = np.zeros((h, w, 4), np.uint8)
        P = C.POINTER
        self.check(lib().mm3e_reproject(self._ptr, w, h, C.byref(gframe["camera"]), color.ctypes.data_as(P(C.c_uint8)),
                                        depth.ctypes.data_as(P(C.c_float)), obj.ctypes.data_as(P(C.c_int32)),
                                        C.byref(new_camera), dl.ctypes.data_as(P(C.c_float)), len(dl),
                                        hybrid_scene._ptr if hybrid_scene is not None else None,
                                        out.ctypes.data_as(P(C.c_uint8))))
        return out

    # ---- mesh -> SDF bake -------------------------------------------------------------------------
    def bake_mesh_sdf(self, positions, triangles, resolution, padding, device_out=None):
        """mesh::bake_sdf on the GPU. Returns an SdfVolume (host samples), or, with `device_out`
        (a device pointer with room for the grid), the grid (dims, min, cell) only."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        tri = np.ascontiguousarray(triangles, np.uint32).reshape(-1)
        m = abi.Mesh(pos.ctypes.data_as(C.POINTER(C.c_float)), len(pos) // 3,
                     tri.ctypes.data_as(C.POINTER(C.c_uint32)), len(tri) // 3)
        v = abi.Volume()
        self.check(lib().mm3e_bake_mesh_sdf(self._ptr, C.byref(m), resolution, padding, C.byref(v), None, 0, 0))
        n = v.nx * v.ny * v.nz
        dims, vmin, cell = (v.nx, v.ny, v.nz), tuple(v.min), tuple(v.cell)
        if device_out is not None:
            self.check(lib().mm3e_bake_mesh_sdf(self._ptr, C.byref(m), resolution, padding, C.byref(v),
                                                C.c_void_p(device_out), n, 1))
            return dims, vmin, cell
        data = np.zeros(n, np.float32)
        self.check(lib().mm3e_bake_mesh_sdf(self._ptr, C.byref(m), resolution, padding, C.byref(v),
                                            data.ctypes.data_as(C.c_void_p), n, 0))
        from .scene import SdfVolume
        return SdfVolume(dims, vmin, cell, data)

    def close(self):
        """Destroy the context; scenes compiled on it are destroyed first."""
        if self._ptr:
            for sc in list(self._scenes):
                sc.close()
            lib().mm3e_ctx_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class CompiledScene:
    """A scene lowered to a device-resident tape (mm3e_scene)."""

    def __init__(self, ctx, scene):
        self.ctx = ctx
        self.width, self.height = scene.width, scene.height
        self.mode = scene.mode
        self.n_materials = len(scene.materials)
        handle = scene.desc()
        self._ptr = C.c_void_p()
        ctx.check(lib().mm3e_scene_compile(ctx.handle, handle.ptr, C.byref(self._ptr)))
        ctx._scenes.add(self)

    def close(self):
        if self._ptr:
            if self.ctx.handle:
                lib().mm3e_scene_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    SPEC_OFF, SPEC_AUTO, SPEC_ALWAYS = 0, 1, 2

    def specialize(self, mode=2):
        """Scene-specialised march / shadow / AO kernels (NVRTC): mode 0 off, 1 auto (only
        fields of at most 64 objects), 2 always (True/False map to 2/0). Returns compile ms."""
        mode = {True: 2, False: 0}.get(mode, mode) if isinstance(mode, bool) else mode
        ms = C.c_double()
        self.ctx.check(lib().mm3e_scene_specialize(self._ptr, int(mode), C.byref(ms)))
        return ms.value

    @property
    def specialized(self):
        return bool(lib().mm3e_scene_is_specialized(self._ptr))

    def device_bytes(self):
        n = C.c_size_t()
        self.ctx.check(lib().mm3e_scene_device_bytes(self._ptr, C.byref(n)))
        return n.value

    def render(self, camera, dyn_spheres=(), fmt=abi.FB_RGBA_F32, stats=False, out=None):
        """Framebuffer of the frame: (h, w, 4) f32 RGBA, or (h, w, 4) u8 for FB_RGBA8; into `out`
        (a C-contiguous array of that shape and type, reused across frames) when given."""
        h, w = self.height, self.width
        dtype = np.float32 if fmt == abi.FB_RGBA_F32 else np.uint8
        if out is None:
            out = np.empty((h, w, 4), dtype=dtype)
        elif out.shape != (h, w, 4) or out.dtype != dtype or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous ({h}, {w}, 4) {np.dtype(dtype).name} array")
        dyn = (abi.DynSphere * max(1, len(dyn_spheres)))(*[s.to_abi() for s in dyn_spheres])
        st = abi.RenderStats()
        rc = lib().mm3e_render(self._ptr, C.byref(camera), dyn, len(dyn_spheres), fmt,
                               out.ctypes.data_as(C.c_void_p), out.nbytes, C.byref(st))
        self.ctx.check(rc)
        if stats:
            return out, {"device_ms": st.device_ms, "total_ms": st.total_ms, "d2h_bytes": st.d2h_bytes,
                         "kernel_launches": st.kernel_launches}
        return out

    # CpuParallelScene::try_render (mm3e-cpu-parallel/src/lib.rs:50-65)
    def try_render(self, camera, dyn_spheres=()):
        return self.render(camera, dyn_spheres)

    def render_linear(self, camera):
        """render_linear: beauty radiance before post, (h, w, 3) f32."""
        out = np.empty((self.height, self.width, 3), dtype=np.float32)
        self.ctx.check(lib().mm3e_render_linear(self._ptr, C.byref(camera),
                                                out.ctypes.data_as(C.POINTER(C.c_float)), out.size))
        return out

    def render_device(self, camera, fmt, device_ptr, nbytes):
        self.ctx.check(lib().mm3e_render_device(self._ptr, C.byref(camera), fmt, C.c_void_p(device_ptr), nbytes))

    def render_hits(self, camera):
        n = self.width * self.height
        t = np.empty(n, np.float32)
        m = np.empty(n, np.uint32)
        s = np.empty(n, np.uint32)
        nrm = np.empty(3 * n, np.float32)
        P = C.POINTER
        self.ctx.check(lib().mm3e_render_hits(self._ptr, C.byref(camera), t.ctypes.data_as(P(C.c_float)),
                                              m.ctypes.data_as(P(C.c_uint32)), s.ctypes.data_as(P(C.c_uint32)),
                                              nrm.ctypes.data_as(P(C.c_float))))
        shape = (self.height, self.width)
        return {"t": t.reshape(shape), "mat": m.reshape(shape), "steps": s.reshape(shape),
                "normal": nrm.reshape(shape + (3,))}

    def render_film(self, camera, aperture_radius=0.0, focus_distance=1.0):
        """render_film: dict of beauty / foreground (h, w, 3), alpha / depth (h, w), normals
        (h, w, 3), material_ids (h, w)."""
        h, w = self.height, self.width
        out = {"beauty": np.zeros((h, w, 3), np.float32), "foreground": np.zeros((h, w, 3), np.float32),
               "alpha": np.zeros((h, w), np.float32), "depth": np.zeros((h, w), np.float32),
               "normals": np.zeros((h, w, 3), np.float32), "material_ids": np.zeros((h, w), np.uint32)}
        P = C.POINTER
        f = lambda a: a.ctypes.data_as(P(C.c_float))
        self.ctx.check(lib().mm3e_render_film(self._ptr, C.byref(camera), aperture_radius, focus_distance,
                                              f(out["beauty"]), f(out["foreground"]), f(out["alpha"]),
                                              f(out["depth"]), f(out["normals"]),
                                              out["material_ids"].ctypes.data_as(P(C.c_uint32))))
        return out

    def autotune(self, camera, spec_mode=1, candidates=None, repeats=5):
        """mm3e_scene_autotune: the fastest launch shape for this scene's frames at `camera` becomes
        the scene's own; returns (best tuning dict, [(tuning dict, median ms)])."""
        cand = None
        n = 0
        if candidates:
            cand = (abi.Tuning * len(candidates))(*[abi.Tuning(c["block"], c["tile_wlog"], c["unroll"],
                                                               c.get("min_blocks", 0)) for c in candidates])
            n = len(candidates)
        best = abi.Tuning()
        rep = (abi.TuneEntry * 64)()
        nr = C.c_uint32()
        self.ctx.check(lib().mm3e_scene_autotune(self._ptr, C.byref(camera), spec_mode, cand, n, repeats, C.byref(best),
                                                 rep, 64, C.byref(nr)))
        as_dict = lambda t: {"block": t.block, "tile_wlog": t.tile_wlog, "unroll": t.unroll, "min_blocks": t.min_blocks}
        return as_dict(best), [(as_dict(rep[i].tuning), rep[i].device_ms) for i in range(nr.value)]

    def render_gbuffer(self, camera, movers=()):
        """render_gbuffer (lib.rs:951): a GFrame dict — color (h, w, 4) u8, depth (h, w) f32 (+inf on
        a miss), obj (h, w) i32 (-1: no mover), camera. `movers`: (centre xyz, radius) per mover."""
        h, w = self.height, self.width
        mv = np.ascontiguousarray(np.asarray(movers, np.float32).reshape(-1, 4))
        out = {"color": np.zeros((h, w, 4), np.uint8), "depth": np.zeros((h, w), np.float32),
               "obj": np.zeros((h, w), np.int32), "camera": camera}
        P = C.POINTER
        self.ctx.check(lib().mm3e_render_gbuffer(self._ptr, C.byref(camera), mv.ctypes.data_as(P(C.c_float)), len(mv),
                                                 out["color"].ctypes.data_as(P(C.c_uint8)),
                                                 out["depth"].ctypes.data_as(P(C.c_float)),
                                                 out["obj"].ctypes.data_as(P(C.c_int32))))
        return out

    def march_rays(self, rays6):
        rays6 = np.ascontiguousarray(rays6, dtype=np.float32).reshape(-1, 6)
        n = len(rays6)
        t = np.empty(n, np.float32)
        m = np.empty(n, np.uint32)
        s = np.empty(n, np.uint32)
        P = C.POINTER
        self.ctx.check(lib().mm3e_march_rays(self._ptr, rays6.ctypes.data_as(P(C.c_float)), n,
                                             t.ctypes.data_as(P(C.c_float)), m.ctypes.data_as(P(C.c_uint32)),
                                             s.ctypes.data_as(P(C.c_uint32))))
        return t, m, s

    def field(self, points3):
        pts = np.ascontiguousarray(points3, dtype=np.float32).reshape(-1, 3)
        n = len(pts)
        d = np.empty(n, np.float32)
        m = np.empty(n, np.uint32)
        P = C.POINTER
        self.ctx.check(lib().mm3e_field(self._ptr, pts.ctypes.data_as(P(C.c_float)), n,
                                        d.ctypes.data_as(P(C.c_float)), m.ctypes.data_as(P(C.c_uint32))))
        return d, m

    def bake_gi(self, dims, samples):
        """Scene::bake_gi on the GPU (replaces the compiled scene's GI)."""
        self.ctx.check(lib().mm3e_bake_gi(self._ptr, dims[0], dims[1], dims[2], samples))

    def get_gi(self):
        mn = (C.c_float * 3)()
        sz = (C.c_float * 3)()
        dims = (C.c_uint32 * 3)()
        self.ctx.check(lib().mm3e_scene_get_gi(self._ptr, mn, sz, dims, None, 0))
        n = dims[0] * dims[1] * dims[2] * 18
        cubes = np.empty(n, np.float32)
        self.ctx.check(lib().mm3e_scene_get_gi(self._ptr, mn, sz, dims, cubes.ctypes.data_as(C.POINTER(C.c_float)),
                                               n))
        return GiVolume(tuple(mn), tuple(sz), tuple(dims), cubes)


class CudaRenderer:
    """CpuParallelRenderer counterpart: compile scenes for one GPU context."""

    def __init__(self, device=0, ctx=None):
        self.ctx = ctx or (default_context() if device == 0 else Context(device))

    def compile(self, scene):
        return CompiledScene(self.ctx, scene)


def spec_source(scene):
    """The generated scene-specialised program (host only)."""
    h = scene.desc()
    n = C.c_size_t()
    lib().mm3e_scene_spec_source(h.ptr, None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value + 1)
    rc = lib().mm3e_scene_spec_source(h.ptr, buf, n.value + 1, C.byref(n))
    if rc != abi.OK:
        raise RenderError(rc, "spec source")
    return buf.value.decode()


def scene_tape(scene):
    """The lowered scene tape (host only): the bytes the device holds for the scene."""
    h = scene.desc()
    n = C.c_size_t()
    rc = lib().mm3e_scene_tape(h.ptr, None, 0, C.byref(n))
    if rc != abi.OK:
        raise RenderError(rc, "scene tape")
    buf = C.create_string_buffer(n.value)
    rc = lib().mm3e_scene_tape(h.ptr, buf, n.value, C.byref(n))
    if rc != abi.OK:
        raise RenderError(rc, "scene tape")
    return buf.raw[:n.value]


def spec_compile_check(scene):
    """NVRTC compile of the scene's specialised program (host only): (ok, message, ms)."""
    h = scene.desc()
    err = C.create_string_buffer(8192)
    ms = C.c_double()
    rc = lib().mm3e_spec_compile_check(h.ptr, err, 8192, C.byref(ms))
    return rc == abi.OK, err.value.decode(errors="replace"), ms.value


def validate(scene):
    """mm3e_scene_validate: (code, message) without touching a GPU."""
    buf = C.create_string_buffer(512)
    h = scene.desc()
    rc = lib().mm3e_scene_validate(h.ptr, buf, len(buf))
    return rc, buf.value.decode(errors="replace")


def render(scene, camera, ctx=None):
    """mm3e_orchestrator::render_checked: compile + render one frame, RGBA f32 (h, w, 4)."""
    return CompiledScene(ctx or default_context(), scene).render(camera)


def render_linear(scene, camera, ctx=None):
    return CompiledScene(ctx or default_context(), scene).render_linear(camera)


def _flatten_u8(fb, background):
    """Straight alpha over `background` and the u8 quantisation of Framebuffer's encoders
    (framebuffer.rs:84-91,103-111,117-125): per channel (clamp(c * a + bg * (1 - a), 0, 1) * 255
    + 0.5) as u8, a = clamp(alpha, 0, 1), every step in binary32; a NaN channel gives 0, as Rust's
    `as u8` does. Returns (..., 3) uint8 RGB."""
    fb = np.asarray(fb, dtype=np.float32)
    bg = np.asarray(background, dtype=np.float32)[:3]
    with np.errstate(invalid="ignore"):
        a = np.clip(fb[..., 3:4], np.float32(0.0), np.float32(1.0)).astype(np.float32)
        rgb = (fb[..., :3] * a + bg * (np.float32(1.0) - a)).astype(np.float32)
        q = (np.clip(rgb, np.float32(0.0), np.float32(1.0)) * np.float32(255.0) + np.float32(0.5)).astype(np.float32)
        q = np.where(np.isnan(q), np.float32(0.0), q)
    return np.floor(q).astype(np.uint8)


def to_rgba8(fb, background=(0.0, 0.0, 0.0, 1.0)):
    """Framebuffer::to_rgba8 (framebuffer.rs:102-113): opaque RGBA8 over `background` (black by
    default) for an (h, w, 4) RGBA f32 frame."""
    rgb = _flatten_u8(fb, background)
    out = np.empty(rgb.shape[:-1] + (4,), np.uint8)
    out[..., :3] = rgb
    out[..., 3] = 255
    return out


def to_u32(fb, background=(0.0, 0.0, 0.0, 1.0)):
    """Framebuffer::to_u32 (framebuffer.rs:115-127): opaque 0x00RRGGBB pixels, (h, w) uint32."""
    rgb = _flatten_u8(fb, background).astype(np.uint32)
    return (rgb[..., 0] << 16) | (rgb[..., 1] << 8) | rgb[..., 2]


def to_bmp(fb, background=(0.0, 0.0, 0.0, 1.0)):
    """Framebuffer::to_bmp (framebuffer.rs:54-99): a 24-bit bottom-up BMP (14-byte file header,
    40-byte info header at 2835 pixels per metre, BGR rows padded to 4 bytes), as bytes."""
    rgb = _flatten_u8(fb, background)
    h, w = rgb.shape[:2]
    pad = (4 - (w * 3) % 4) % 4
    row_bytes = w * 3 + pad
    pixel_bytes = row_bytes * h
    file_size = 54 + pixel_bytes
    if file_size > 0xFFFFFFFF:
        raise ValueError("BMP file too large for 32-bit BMP header")
    header = (b"BM" + np.array([file_size, 0, 54, 40], "<u4").tobytes() + np.array([w, h], "<i4").tobytes() +
              np.array([1, 24], "<u2").tobytes() + np.array([0, pixel_bytes], "<u4").tobytes() +
              np.array([2835, 2835], "<i4").tobytes() + np.array([0, 0], "<u4").tobytes())
    rows = np.zeros((h, row_bytes), np.uint8)
    rows[:, :w * 3] = rgb[::-1, :, ::-1].reshape(h, w * 3)
    return header + rows.tobytes()


__all__ = [
    "abi", "lib", "NativeLibraryMissing", "RenderError", "Context", "CompiledScene", "CudaRenderer", "render",
    "render_linear", "validate", "to_rgba8", "to_u32", "to_bmp", "Scene", "Object", "Prim", "Material", "Light", "directional", "Marcher",
    "Post", "Transform", "Expr", "SdfVolume", "GiVolume", "DynSphere", "look_at", "orbit_camera", "mat3_from_euler",
    "quat_to_mat3", "normalize_f32", "radians",
]


class Server:
    """The served form (mm3e_server): continuous batching of render requests on one GPU.

    While a server runs on a Context, use the context only through the server."""

    def __init__(self, ctx, hbm_budget_bytes=0, max_samples=0, max_inflight=0, use_graphs=True, plain=False,
                 spec_workers=0):
        self.ctx = ctx
        self._ptr = C.c_void_p()
        self._keep = {}  # request inputs that must outlive submission (ticket -> objects)
        cfg = abi.ServerConfig(hbm_budget_bytes, max_samples, max_inflight, 1 if use_graphs else 0, 1 if plain else 0,
                               int(spec_workers))
        ctx.check(lib().mm3e_server_create(ctx.handle, C.byref(cfg), C.byref(self._ptr)))

    def add_scene(self, scene):
        sid = C.c_uint32()
        h = scene.desc()
        self.ctx.check(lib().mm3e_server_add_scene(self._ptr, h.ptr, C.byref(sid)))
        return sid.value

    @staticmethod
    def request(camera, out, scene_id=0, new_scene=None, mesh=None, mesh_volume=0, mesh_resolution=128,
                mesh_padding=0.1, width=0, height=0, fmt=abi.FB_RGBA8):
        """A Request struct plus the objects it points to (keep them alive until completion).
        `out`: host ndarray for the frame; `new_scene`: Scene; `mesh`: (positions, triangles)."""
        r = abi.Request()
        keep = [out]
        r.scene_id = scene_id
        if new_scene is not None:
            h = new_scene.desc()
            keep.append(h)
            r.new_scene = C.pointer(h.desc)
        if mesh is not None:
            pos = np.ascontiguousarray(mesh[0], np.float32).reshape(-1)
            tri = np.ascontiguousarray(mesh[1], np.uint32).reshape(-1)
            m = abi.Mesh(pos.ctypes.data_as(C.POINTER(C.c_float)), len(pos) // 3,
                         tri.ctypes.data_as(C.POINTER(C.c_uint32)), len(tri) // 3)
            keep += [pos, tri, m]
            r.mesh = C.pointer(m)
            r.mesh_volume, r.mesh_resolution, r.mesh_padding = mesh_volume, mesh_resolution, mesh_padding
        r.camera = camera
        r.width, r.height, r.format = width, height, fmt
        r.host_out = out.ctypes.data
        r.out_bytes = out.nbytes
        return r, keep

    def submit(self, req, keep=None):
        t = C.c_uint64()
        self.ctx.check(lib().mm3e_server_submit(self._ptr, C.byref(req), C.byref(t)))
        return t.value

    def wait(self, ticket, timeout_ms=0):
        res = abi.RequestResult()
        rc = lib().mm3e_server_wait(self._ptr, ticket, timeout_ms, C.byref(res))
        if rc == abi.ERR_BUSY:
            return None
        return {"status": res.status, "scene_id": res.scene_id, "submit_ms": res.submit_ms,
                "start_ms": res.start_ms, "done_ms": res.done_ms}

    def stats(self):
        st = abi.ServerStats()
        self.ctx.check(lib().mm3e_server_get_stats(self._ptr, C.byref(st)))
        return {k: getattr(st, k) for k, _ in abi.ServerStats._fields_}

    def replay(self, requests, arrivals_s):
        """Open-loop replay of a Request array at the given arrival times (seconds)."""
        n = len(requests)
        arr = (abi.Request * n)(*requests)
        times = (C.c_double * n)(*arrivals_s)
        res = (abi.RequestResult * n)()
        rc = lib().mm3e_server_replay(self._ptr, arr, times, n, res)
        out = [{"status": r.status, "scene_id": r.scene_id, "submit_ms": r.submit_ms, "start_ms": r.start_ms,
                "done_ms": r.done_ms} for r in res]
        return rc, out

    def close(self):
        if self._ptr:
            lib().mm3e_server_destroy(self._ptr)
            self._ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
