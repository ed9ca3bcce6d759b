"""Python binding of the CPU oracle (liboracle_mm3e.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, as the checker or the timed CPU reference. It takes the same scene descriptions
(`Scene.desc()`) and cameras as the CUDA library.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None
P = C.POINTER


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        l = C.CDLL(path)
        vp = C.c_void_p
        l.oracle_render.argtypes = [vp, vp, C.c_uint, P(C.c_float), P(C.c_float)]
        l.oracle_render_rows.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint, P(C.c_float)]
        l.oracle_post.argtypes = [vp, P(C.c_float), P(C.c_float)]
        l.oracle_primary_hits.argtypes = [vp, vp, C.c_uint, P(C.c_float), P(C.c_uint32), P(C.c_uint32), P(C.c_float)]
        l.oracle_march_rays.argtypes = [vp, P(C.c_float), C.c_size_t, C.c_int, C.c_uint, P(C.c_double),
                                        P(C.c_uint32), P(C.c_uint32), P(C.c_double)]
        l.oracle_soft_shadows.argtypes = [vp, P(C.c_float), C.c_size_t, C.c_uint, P(C.c_float)]
        l.oracle_ambient_occlusion.argtypes = [vp, P(C.c_float), C.c_size_t, C.c_uint, P(C.c_float)]
        l.oracle_sdf.argtypes = [C.c_uint32, P(C.c_float), C.c_float, C.c_float, C.c_float]
        l.oracle_sdf.restype = C.c_float
        l.oracle_combine.argtypes = [C.c_uint32, C.c_float, C.c_uint32, C.c_float, C.c_uint32, C.c_float,
                                     P(C.c_float), P(C.c_uint32)]
        l.oracle_domain.argtypes = [C.c_uint32, P(C.c_float), C.c_float, C.c_float, C.c_float]
        l.oracle_brdf.argtypes = [P(C.c_float)] * 4 + [C.c_float, C.c_float, C.c_float, P(C.c_float)]
        l.oracle_fresnel.argtypes = [C.c_float, C.c_float]
        l.oracle_fresnel.restype = C.c_float
        l.oracle_aces.argtypes = [P(C.c_float), P(C.c_float)]
        l.oracle_field.argtypes = [vp, P(C.c_float), C.c_size_t, C.c_int, P(C.c_float), P(C.c_uint32)]
        l.oracle_count_frame.argtypes = [vp, vp, C.c_uint, P(C.c_uint64)]
        l.oracle_bake_mesh_sdf.argtypes = [P(C.c_float), C.c_uint32, P(C.c_uint32), C.c_uint32, C.c_uint32, C.c_float,
                                           C.c_uint, P(C.c_uint32), P(C.c_float), P(C.c_float), P(C.c_float),
                                           C.c_size_t, C.c_char_p, C.c_size_t]
        l.oracle_x_crossing.argtypes = [P(C.c_float), P(C.c_float), P(C.c_float), C.c_float, C.c_float, P(C.c_float)]
        l.oracle_render_film.argtypes = [vp, vp, C.c_float, C.c_float, C.c_uint, P(C.c_float), P(C.c_float),
                                         P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_uint32)]
        u8p = P(C.c_uint8)
        l.oracle_render_gbuffer.argtypes = [vp, vp, P(C.c_float), C.c_uint32, C.c_uint, u8p, P(C.c_float),
                                            P(C.c_int32)]
        l.oracle_reproject_warp.argtypes = [C.c_uint32, C.c_uint32, vp, u8p, P(C.c_float), P(C.c_int32), vp,
                                            P(C.c_float), C.c_uint32, u8p, u8p]
        l.oracle_reproject_fill.argtypes = [C.c_uint32, C.c_uint32, u8p, u8p]
        l.oracle_rerender_holes.argtypes = [vp, vp, C.c_uint, u8p, u8p]
        l.oracle_count_frame_blocks.argtypes = [vp, vp, C.c_uint, P(C.c_uint64), C.c_int]
        l.oracle_bake_gi.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint, P(C.c_float),
                                     P(C.c_float), P(C.c_uint32), P(C.c_float)]
        l.oracle_gi_sample.argtypes = [vp, P(C.c_float), P(C.c_float), C.c_size_t, P(C.c_float)]
        l.oracle_time_rows.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint]
        l.oracle_time_rows.restype = C.c_double
        l.oracle_camera_look_at.argtypes = [P(C.c_float), P(C.c_float), P(C.c_float), C.c_float, vp]
        l.oracle_orbit_camera.argtypes = [P(C.c_float), C.c_float, C.c_float, C.c_float, C.c_float, vp]
        l.oracle_mat3_from_euler.argtypes = [C.c_float, C.c_float, C.c_float, P(C.c_float)]
        l.oracle_quat_to_mat3.argtypes = [P(C.c_float), P(C.c_float)]
        _lib = l
    return _lib


def threads_default():
    return os.cpu_count() or 1


def _f(a):
    return a.ctypes.data_as(P(C.c_float))


def render(handle, cam, threads=None, want_hdr=False):
    """Reference render(): RGBA f32 framebuffer (h, w, 4) [, HDR (h, w, 3)]."""
    d = handle.desc
    h, w = d.height, d.width
    rgba = np.zeros((h, w, 4), np.float32)
    hdr = np.zeros((h, w, 3), np.float32) if want_hdr else None
    rc = lib().oracle_render(C.addressof(d), C.addressof(cam), threads or threads_default(), _f(rgba),
                             _f(hdr) if want_hdr else None)
    if rc != 0:
        raise RuntimeError(f"oracle_render failed ({rc})")
    return (rgba, hdr) if want_hdr else rgba


def render_rows(handle, cam, y0, y1, threads=None):
    d = handle.desc
    out = np.zeros((y1 - y0, d.width, 3), np.float32)
    rc = lib().oracle_render_rows(C.addressof(d), C.addressof(cam), y0, y1, threads or threads_default(), _f(out))
    if rc != 0:
        raise RuntimeError("oracle_render_rows failed")
    return out


def post(handle, hdr):
    d = handle.desc
    hdr = np.ascontiguousarray(hdr, np.float32)
    rgba = np.zeros((d.height, d.width, 4), np.float32)
    lib().oracle_post(C.addressof(d), _f(hdr), _f(rgba))
    return rgba


def primary_hits(handle, cam, threads=None):
    d = handle.desc
    n = d.width * d.height
    t = np.zeros(n, np.float32)
    m = np.zeros(n, np.uint32)
    s = np.zeros(n, np.uint32)
    nrm = np.zeros(3 * n, np.float32)
    lib().oracle_primary_hits(C.addressof(d), C.addressof(cam), threads or threads_default(), _f(t),
                              m.ctypes.data_as(P(C.c_uint32)), s.ctypes.data_as(P(C.c_uint32)), _f(nrm))
    shape = (d.height, d.width)
    return {"t": t.reshape(shape), "mat": m.reshape(shape), "steps": s.reshape(shape),
            "normal": nrm.reshape(shape + (3,))}


def march_rays(handle, rays6, use_double=False, threads=None, normals=False):
    rays6 = np.ascontiguousarray(rays6, np.float32).reshape(-1, 6)
    n = len(rays6)
    t = np.zeros(n, np.float64)
    m = np.zeros(n, np.uint32)
    s = np.zeros(n, np.uint32)
    nrm = np.zeros(3 * n, np.float64) if normals else None
    lib().oracle_march_rays(C.addressof(handle.desc), _f(rays6), n, 1 if use_double else 0, threads or threads_default(),
                            t.ctypes.data_as(P(C.c_double)), m.ctypes.data_as(P(C.c_uint32)),
                            s.ctypes.data_as(P(C.c_uint32)),
                            nrm.ctypes.data_as(P(C.c_double)) if normals else None)
    if normals:
        return t, m, s, nrm.reshape(n, 3)
    return t, m, s


def soft_shadows(handle, rays6, threads=None):
    """Soft-shadow factor of every (ray, light) at the ray's binary32 hit, shape (n, n_lights);
    -1 where no shadow ray is cast."""
    rays6 = np.ascontiguousarray(rays6, np.float32).reshape(-1, 6)
    n, nl = len(rays6), handle.desc.n_lights
    out = np.zeros(max(n * nl, 1), np.float32)
    lib().oracle_soft_shadows(C.addressof(handle.desc), _f(rays6), n, threads or threads_default(), _f(out))
    return out[:n * nl].reshape(n, nl)


def ambient_occlusion(handle, rays6, threads=None):
    """Ambient occlusion at every ray's binary32 hit; -1 on a miss or with AO off."""
    rays6 = np.ascontiguousarray(rays6, np.float32).reshape(-1, 6)
    out = np.zeros(max(len(rays6), 1), np.float32)
    lib().oracle_ambient_occlusion(C.addressof(handle.desc), _f(rays6), len(rays6), threads or threads_default(), _f(out))
    return out[:len(rays6)]


def sdf(kind, params, p):
    q = (C.c_float * 7)(*(list(params) + [0.0] * (7 - len(params))))
    return lib().oracle_sdf(kind, q, p[0], p[1], p[2])


def combine(op, a, b, k=0.0):
    """a, b = (dist, mat); op 0 union, 1 intersect, 2 subtract, 3 smooth_union, 4 smooth_subtract,
    5 smooth_intersect."""
    d = C.c_float()
    m = C.c_uint32()
    lib().oracle_combine(op, a[0], a[1], b[0], b[1], k, C.byref(d), C.byref(m))
    return d.value, m.value


def domain(op, p, a=0.0, b=0.0, c=0.0):
    v = (C.c_float * 3)(*p)
    lib().oracle_domain(op, v, a, b, c)
    return tuple(v)


def brdf(n, l, v, albedo, metallic, roughness, reflectance):
    out = (C.c_float * 3)()
    F3 = C.c_float * 3
    lib().oracle_brdf(F3(*n), F3(*l), F3(*v), F3(*albedo), metallic, roughness, reflectance, out)
    return tuple(out)


def fresnel(c, f0):
    return lib().oracle_fresnel(c, f0)


def aces(x):
    out = (C.c_float * 3)()
    lib().oracle_aces((C.c_float * 3)(*x), out)
    return tuple(out)


def field(handle, pts, linear=False):
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    d = np.zeros(len(pts), np.float32)
    m = np.zeros(len(pts), np.uint32)
    lib().oracle_field(C.addressof(handle.desc), _f(pts), len(pts), 1 if linear else 0, _f(d),
                       m.ctypes.data_as(P(C.c_uint32)))
    return d, m


COUNT_KEYS = ["fp32", "add", "mul", "cmp", "minmax", "div", "sqrt", "trans", "field_evals", "dual_evals",
              "primary_rays", "reflection_rays", "shadow_rays", "gi_rays"]


COUNT_BLOCKS = ("render", "post", "march", "ao", "shadow", "shade", "march_refl", "ao_refl", "shadow_refl")


def count_frame(handle, cam, threads=None):
    """Algorithmic work of one frame (f32 op counts, rays): {"render", "post"} plus the render
    phase split by kernel ("march" incl. hit normals, "ao", "shadow" of the primary level,
    "shade" of all levels, "march_refl", "ao_refl", "shadow_refl" of the reflection levels)."""
    out = (C.c_uint64 * (14 * len(COUNT_BLOCKS)))()
    lib().oracle_count_frame_blocks(C.addressof(handle.desc), C.addressof(cam), threads or threads_default(), out,
                                    len(COUNT_BLOCKS))
    vals = [int(v) for v in out]
    return {name: dict(zip(COUNT_KEYS, vals[14 * i:14 * i + 14])) for i, name in enumerate(COUNT_BLOCKS)}


def bake_gi(handle, dims, samples, threads=None):
    """Scene::bake_gi on the CPU: (min, size, dims, cubes[n*18]) or None if nothing is bounded."""
    mn = np.zeros(3, np.float32)
    sz = np.zeros(3, np.float32)
    dd = np.zeros(3, np.uint32)
    n = max(1, dims[0]) * max(1, dims[1]) * max(1, dims[2])
    cubes = np.zeros(n * 18, np.float32)
    rc = lib().oracle_bake_gi(C.addressof(handle.desc), dims[0], dims[1], dims[2], samples,
                              threads or threads_default(), _f(mn), _f(sz), dd.ctypes.data_as(P(C.c_uint32)), _f(cubes))
    if rc == 0:
        return None
    return tuple(mn), tuple(sz), tuple(int(x) for x in dd), cubes


def gi_sample(handle, pts, nrm):
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    nrm = np.ascontiguousarray(nrm, np.float32).reshape(-1, 3)
    out = np.zeros_like(pts)
    rc = lib().oracle_gi_sample(C.addressof(handle.desc), _f(pts), _f(nrm), len(pts), _f(out))
    if rc != 0:
        raise RuntimeError("scene has no GI")
    return out


def time_rows(handle, cam, y0, y1, threads=None):
    return lib().oracle_time_rows(C.addressof(handle.desc), C.addressof(cam), y0, y1, threads or threads_default())


def bake_mesh_sdf(positions, triangles, resolution, padding, threads=None, grid_only=False):
    """mesh.rs bake_sdf: (dims (nx, ny, nz), min, cell, data (nz, ny, nx) or None). Raises
    ValueError with the reference's message on invalid input."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
    tri = np.ascontiguousarray(triangles, np.uint32).reshape(-1)
    dims = np.zeros(3, np.uint32)
    mn = np.zeros(3, np.float32)
    cell = np.zeros(3, np.float32)
    err = C.create_string_buffer(256)
    l = lib()
    rc = l.oracle_bake_mesh_sdf(_f(pos), len(pos) // 3, tri.ctypes.data_as(P(C.c_uint32)), len(tri) // 3,
                                resolution, padding, threads or threads_default(),
                                dims.ctypes.data_as(P(C.c_uint32)), _f(mn), _f(cell), None, 0, err, 256)
    if rc != 0:
        raise ValueError(err.value.decode())
    if grid_only:
        return tuple(int(d) for d in dims), mn, cell, None
    data = np.zeros(int(dims[0]) * int(dims[1]) * int(dims[2]), np.float32)
    rc = l.oracle_bake_mesh_sdf(_f(pos), len(pos) // 3, tri.ctypes.data_as(P(C.c_uint32)), len(tri) // 3,
                                resolution, padding, threads or threads_default(),
                                dims.ctypes.data_as(P(C.c_uint32)), _f(mn), _f(cell), _f(data), data.size, err, 256)
    if rc != 0:
        raise ValueError(err.value.decode())
    return tuple(int(d) for d in dims), mn, cell, data.reshape(int(dims[2]), int(dims[1]), int(dims[0]))


def x_crossing(a, b, c, y, z):
    """triangle.rs x_crossing: the crossing x (float) or None."""
    x = C.c_float()
    fa, fb, fc = (np.ascontiguousarray(v, np.float32) for v in (a, b, c))
    ok = lib().oracle_x_crossing(_f(fa), _f(fb), _f(fc), y, z, C.byref(x))
    return x.value if ok else None


def render_film(handle, cam, aperture_radius=0.0, focus_distance=1.0, threads=None):
    """film.rs render_film: dict of beauty (h, w, 3), foreground (h, w, 3), alpha, depth (h, w),
    normals (h, w, 3), material_ids (h, w)."""
    d = handle.desc
    h, w = d.height, d.width
    out = {"beauty": np.zeros((h, w, 3), np.float32), "foreground": np.zeros((h, w, 3), np.float32),
           "alpha": np.zeros((h, w), np.float32), "depth": np.zeros((h, w), np.float32),
           "normals": np.zeros((h, w, 3), np.float32), "material_ids": np.zeros((h, w), np.uint32)}
    rc = lib().oracle_render_film(C.addressof(d), C.addressof(cam), aperture_radius, focus_distance,
                                  threads or threads_default(), _f(out["beauty"]), _f(out["foreground"]),
                                  _f(out["alpha"]), _f(out["depth"]), _f(out["normals"]),
                                  out["material_ids"].ctypes.data_as(P(C.c_uint32)))
    if rc != 0:
        raise ValueError("invalid thin lens")
    return out


def _u8(a):
    return a.ctypes.data_as(P(C.c_uint8))


def render_gbuffer(handle, cam, movers=(), threads=None):
    """render_gbuffer: {"color": (h, w, 4) u8, "depth": (h, w) f32, "obj": (h, w) i32}."""
    d = handle.desc
    h, w = d.height, d.width
    mv = np.ascontiguousarray(np.asarray(movers, np.float32).reshape(-1, 4))
    out = {"color": np.zeros((h, w, 4), np.uint8), "depth": np.zeros((h, w), np.float32),
           "obj": np.zeros((h, w), np.int32)}
    lib().oracle_render_gbuffer(C.addressof(d), C.addressof(cam), _f(mv), len(mv), threads or threads_default(),
                                _u8(out["color"]), _f(out["depth"]), out["obj"].ctypes.data_as(P(C.c_int32)))
    return out


def reproject_filled(g, prev_cam, new_cam, deltas=()):
    """reproject::warp's filled mask (reproject.rs:77-113): (h, w) u8, 0 where a hole."""
    h, w = g["depth"].shape
    dl = np.ascontiguousarray(np.asarray(deltas, np.float32).reshape(-1, 3))
    out = np.zeros((h, w, 4), np.uint8)
    filled = np.zeros((h, w), np.uint8)
    lib().oracle_reproject_warp(w, h, C.addressof(prev_cam), _u8(np.ascontiguousarray(g["color"])),
                                _f(np.ascontiguousarray(g["depth"])),
                                np.ascontiguousarray(g["obj"]).ctypes.data_as(P(C.c_int32)), C.addressof(new_cam),
                                _f(dl), len(dl), _u8(out), _u8(filled))
    return filled


def reproject(g, prev_cam, new_cam, deltas=(), hybrid_handle=None, threads=None):
    """reproject::reproject (cheap row fill) or, with hybrid_handle (the scene), reproject_hybrid:
    (h, w, 4) u8."""
    h, w = g["depth"].shape
    dl = np.ascontiguousarray(np.asarray(deltas, np.float32).reshape(-1, 3))
    out = np.zeros((h, w, 4), np.uint8)
    filled = np.zeros((h, w), np.uint8)
    color = np.ascontiguousarray(g["color"])
    lib().oracle_reproject_warp(w, h, C.addressof(prev_cam), _u8(color), _f(np.ascontiguousarray(g["depth"])),
                                np.ascontiguousarray(g["obj"]).ctypes.data_as(P(C.c_int32)), C.addressof(new_cam),
                                _f(dl), len(dl), _u8(out), _u8(filled))
    if hybrid_handle is None:
        lib().oracle_reproject_fill(w, h, _u8(out), _u8(filled))
    else:
        lib().oracle_rerender_holes(C.addressof(hybrid_handle.desc), C.addressof(new_cam), threads or threads_default(),
                                    _u8(out), _u8(filled))
    return out


class HostMath:
    """The oracle's restatements of the reference's scene-building helpers (Camera::look_at,
    orbit_camera, Mat3::from_euler, Quat::to_mat3), with the signatures of the CUDA library's
    host helpers. `mm3e_cuda.scene.use_host_math(HostMath())` builds scenes and cameras through
    them, so that a CPU-only process (the timed reference arm) never loads the CUDA library."""

    @staticmethod
    def camera_look_at(eye3, target3, up3, fov_y, cam_ref):
        lib().oracle_camera_look_at(eye3, target3, up3, fov_y, cam_ref)

    @staticmethod
    def orbit_camera(target3, radius, yaw, pitch, fov_y, cam_ref):
        lib().oracle_orbit_camera(target3, radius, yaw, pitch, fov_y, cam_ref)

    @staticmethod
    def mat3_from_euler(x, y, z, out9):
        lib().oracle_mat3_from_euler(x, y, z, out9)

    @staticmethod
    def quat_to_mat3(q4, out9):
        lib().oracle_quat_to_mat3(q4, out9)
