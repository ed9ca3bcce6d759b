"""Host-side mirror of MM3E's scene API (mm3e_orchestrator::{Scene, Object, Prim, Light},
mm3e_kit::{Material, Marcher, Camera, csg::Expr, volume::SdfVolume}, gi::GiVolume, post::Post).

Names, defaults and argument meaning follow the reference so that scenes written against it
read the same here; `Scene.desc()` marshals the scene into the flat `mm3e_scene_desc` of the
C ABI. All scalar arithmetic that the reference performs while *building* a scene (vector
normalisation, Euler rotations, look-at frames) is done in IEEE binary32, either with numpy
float32 or through the library's host helpers, so the description holds the same f32 values
the Rust constructors would produce.
"""
import copy as _copy
import ctypes as C
import math

import numpy as np

from . import abi
from .native import lib

F32 = np.float32


def _f3(v):
    return tuple(float(F32(x)) for x in v)


def normalize_f32(v):
    """Vec3::normalize (mm3e-kit/src/vec.rs:37-44) in binary32."""
    x, y, z = (F32(c) for c in v)
    ln = np.sqrt(F32(F32(x * x + y * y) + z * z), dtype=F32)
    if ln > F32(1e-12):
        inv = F32(F32(1.0) / ln)
        return (float(x * inv), float(y * inv), float(z * inv))
    return (0.0, 0.0, 0.0)


IDENTITY_ROT = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)


class _LibraryHostMath:
    """The library's own host helpers (libmm3e_cuda.so): the default provider."""

    @staticmethod
    def camera_look_at(eye3, target3, up3, fov_y, cam_ref):
        lib().mm3e_camera_look_at(eye3, target3, up3, fov_y, cam_ref)

    @staticmethod
    def orbit_camera(target3, radius, yaw, pitch, fov_y, cam_ref):
        lib().mm3e_orbit_camera(target3, radius, yaw, pitch, fov_y, cam_ref)

    @staticmethod
    def mat3_from_euler(x, y, z, out9):
        lib().mm3e_mat3_from_euler(x, y, z, out9)

    @staticmethod
    def quat_to_mat3(q4, out9):
        lib().mm3e_quat_to_mat3(q4, out9)


_host_math = _LibraryHostMath()


def use_host_math(provider=None):
    """Route the binary32 scene-building helpers (look_at, orbit_camera, mat3_from_euler,
    quat_to_mat3) through `provider`, an object with the four functions of _LibraryHostMath
    that writes the same values; None restores the library's helpers. A process that must not
    load libmm3e_cuda.so (a CPU-only timing of the reference path) builds its scenes this way.
    Returns the previous provider."""
    global _host_math
    prev = _host_math
    _host_math = provider if provider is not None else _LibraryHostMath()
    return prev


def mat3_from_euler(x, y, z):
    """Mat3::from_euler (vec.rs:144-149): columns as a 9-tuple."""
    out = (C.c_float * 9)()
    _host_math.mat3_from_euler(x, y, z, out)
    return tuple(out)


def quat_to_mat3(q_xyzw):
    """Quat::to_mat3 (vec.rs:318-326)."""
    out = (C.c_float * 9)()
    _host_math.quat_to_mat3((C.c_float * 4)(*q_xyzw), out)
    return tuple(out)


def radians(deg):
    """f32::to_radians: deg * (PI / 180) in binary32."""
    return float(F32(deg) * F32(F32(math.pi) / F32(180.0)))


class Transform:
    """vec.rs:165-222 rigid transform + uniform scale."""

    def __init__(self, pos=(0.0, 0.0, 0.0), rot=IDENTITY_ROT, scale=1.0):
        self.pos = _f3(pos)
        self.rot = tuple(float(F32(r)) for r in rot)
        self.scale = float(F32(scale))

    @staticmethod
    def at(pos):
        return Transform(pos)

    def rotated(self, rot):
        t = _copy.copy(self)
        t.rot = tuple(float(F32(r)) for r in rot)
        return t

    def scaled(self, s):
        t = _copy.copy(self)
        t.scale = float(F32(s))
        return t


Transform.IDENTITY = Transform()


class Prim:
    """lib.rs:157-212 primitive shapes (local space)."""

    def __init__(self, kind, params=(), pid=0):
        self.kind = kind
        self.params = tuple(float(F32(p)) for p in params) + (0.0,) * (7 - len(params))
        self.id = pid

    sphere = staticmethod(lambda r: Prim(abi.PRIM_SPHERE, (r,)))
    box = staticmethod(lambda half: Prim(abi.PRIM_BOX, tuple(half)))
    round_box = staticmethod(lambda half, radius: Prim(abi.PRIM_ROUND_BOX, tuple(half) + (radius,)))
    torus = staticmethod(lambda major, minor: Prim(abi.PRIM_TORUS, (major, minor)))
    cylinder = staticmethod(lambda h, r: Prim(abi.PRIM_CYLINDER, (h, r)))
    capsule = staticmethod(lambda a, b, r: Prim(abi.PRIM_CAPSULE, tuple(a) + tuple(b) + (r,)))
    cone = staticmethod(lambda r1, r2, h: Prim(abi.PRIM_CONE, (r1, r2, h)))
    ellipsoid = staticmethod(lambda r: Prim(abi.PRIM_ELLIPSOID, tuple(r)))
    octahedron = staticmethod(lambda s: Prim(abi.PRIM_OCTAHEDRON, (s,)))
    hex_prism = staticmethod(lambda r, h: Prim(abi.PRIM_HEX_PRISM, (r, h)))
    plane = staticmethod(lambda n, h: Prim(abi.PRIM_PLANE, tuple(n) + (h,)))
    csg = staticmethod(lambda i: Prim(abi.PRIM_CSG, (), i))
    volume = staticmethod(lambda i: Prim(abi.PRIM_VOLUME, (), i))
    surface = staticmethod(lambda i: Prim(abi.PRIM_SURFACE, (), i))


class Object:
    """lib.rs:330-378 a placed object with its combine mode and domain modifiers."""

    def __init__(self, prim, xform, mat):
        self.prim = prim
        self.xform = xform
        self.mat = int(mat)
        self.combine = abi.COMBINE_UNION
        self.k = 0.0
        self.mirror_ = (False, False, False)
        self.repeat_ = (0.0, 0.0, 0.0)
        self.twist_ = 0.0
        self.bend_ = 0.0
        self.elongate_ = (0.0, 0.0, 0.0)
        self.round_ = 0.0
        self.onion_ = 0.0

    def _with(self, **kw):
        o = _copy.copy(self)
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def smooth(self, k):
        return self._with(combine=abi.COMBINE_SMOOTH, k=float(F32(k)))

    def subtract(self):
        return self._with(combine=abi.COMBINE_SUBTRACT)

    def mirror(self, x, y, z):
        return self._with(mirror_=(bool(x), bool(y), bool(z)))

    def repeat(self, period):
        return self._with(repeat_=_f3(period))

    def twist(self, k):
        return self._with(twist_=float(F32(k)))

    def bend(self, k):
        return self._with(bend_=float(F32(k)))

    def elongate(self, h):
        return self._with(elongate_=_f3(h))

    def round(self, r):
        return self._with(round_=float(F32(r)))

    def onion(self, t):
        return self._with(onion_=float(F32(t)))

    def to_abi(self):
        o = abi.Object()
        o.prim = self.prim.kind
        o.id = self.prim.id
        o.mat = self.mat
        o.combine = self.combine
        o.smooth_k = self.k
        o.params[:] = self.prim.params
        o.rot[:] = self.xform.rot
        o.pos[:] = self.xform.pos
        o.scale = self.xform.scale
        o.mirror = (1 if self.mirror_[0] else 0) | (2 if self.mirror_[1] else 0) | (4 if self.mirror_[2] else 0)
        o.repeat[:] = self.repeat_
        o.twist = self.twist_
        o.bend = self.bend_
        o.elongate[:] = self.elongate_
        o.round = self.round_
        o.onion = self.onion_
        return o


class Material:
    """mm3e-kit/src/color.rs:153-206 (defaults from Material::default)."""

    def __init__(self, albedo=(0.8, 0.8, 0.8), metallic=0.0, specular=0.5, roughness=0.35, reflectivity=0.0,
                 emissive=(0.0, 0.0, 0.0), checker=False):
        self.albedo = _f3(albedo)
        self.metallic = float(F32(metallic))
        self.specular = float(F32(specular))
        self.roughness = float(F32(roughness))
        self.reflectivity = float(F32(reflectivity))
        self.emissive = _f3(emissive)
        self.checker = bool(checker)

    @staticmethod
    def solid(albedo, **kw):
        return Material(albedo=albedo, **kw)

    def to_abi(self):
        m = abi.Material()
        m.albedo[:] = self.albedo
        m.metallic = self.metallic
        m.specular = self.specular
        m.roughness = self.roughness
        m.reflectivity = self.reflectivity
        m.emissive[:] = self.emissive
        m.checker = 1 if self.checker else 0
        return m


class Light:
    """lib.rs:503-557."""

    def __init__(self, vec, color, directional, radius=0.0):
        self.vec = _f3(vec)
        self.color = _f3(color)
        self.directional = bool(directional)
        self.radius = float(F32(radius))

    @staticmethod
    def directional_(toward, color):
        return Light(normalize_f32(toward), color, True)

    @staticmethod
    def point(pos, color):
        return Light(pos, color, False)

    @staticmethod
    def sphere(pos, color, radius):
        return Light(pos, color, False, radius)

    def soft(self, radius):
        l = _copy.copy(self)
        l.radius = float(F32(radius))
        return l

    def to_abi(self):
        l = abi.Light()
        l.vec[:] = self.vec
        l.color[:] = self.color
        l.directional = 1 if self.directional else 0
        l.radius = self.radius
        return l


# Rust names `Light::directional`; `directional` is also the field name, so the constructor is
# exposed under both spellings at module level.
def directional(toward, color):
    return Light.directional_(toward, color)


class Marcher:
    """mm3e-kit/src/march.rs:81-96 defaults."""

    def __init__(self):
        self.max_steps = 160
        self.max_dist = 120.0
        self.eps = float(F32(0.0006))
        self.step_scale = 1.0
        self.shadow_steps = 64
        self.ao_samples = 5
        self.lod_footprint = 0.0
        self.subitize = 0.0
        self.secant = False
        self.normal_h = float(F32(0.0009))

    def to_abi(self):
        m = abi.Marcher()
        for k in ("max_steps", "shadow_steps", "ao_samples"):
            setattr(m, k, int(getattr(self, k)))
        for k in ("max_dist", "eps", "step_scale", "lod_footprint", "subitize", "normal_h"):
            setattr(m, k, float(getattr(self, k)))
        m.secant = 1 if self.secant else 0
        return m


class Post:
    """post.rs:25-29 defaults."""

    def __init__(self):
        self.exposure = 1.0
        self.bloom = True
        self.bloom_threshold = 1.0
        self.bloom_intensity = float(F32(0.06))
        self.bloom_radius = 12

    def to_abi(self):
        p = abi.Post()
        p.exposure = self.exposure
        p.bloom = 1 if self.bloom else 0
        p.bloom_threshold = self.bloom_threshold
        p.bloom_intensity = self.bloom_intensity
        p.bloom_radius = int(self.bloom_radius)
        return p


class SdfVolume:
    """mm3e-kit/src/volume.rs:14-23; data row-major (k*ny + j)*nx + i."""

    def __init__(self, dims, vmin, cell, data):
        self.dims = tuple(int(d) for d in dims)
        self.min = _f3(vmin)
        self.cell = _f3(cell)
        self.data = np.ascontiguousarray(data, dtype=F32).reshape(-1)
        if len(self.data) != self.dims[0] * self.dims[1] * self.dims[2]:
            raise ValueError("SdfVolume data length does not match dims")

    def max_cell(self):
        return max(F32(self.cell[0]), F32(self.cell[1]), F32(self.cell[2]))

    def recommended_normal_h(self):
        return float(F32(self.max_cell() * F32(0.6)))

    SDFV_MAGIC = b"MM3ESDF1"

    def to_sdfv_bytes(self):
        """volume.rs:119-137 `.sdfv` cache format (the library's writer)."""
        from .scene_io import serialize_sdfv
        return serialize_sdfv(self)

    @staticmethod
    def from_sdfv_bytes(b):
        """volume.rs:140-176 (the library's parser); SceneFormatError (a ValueError) on bad input."""
        from .scene_io import parse_sdfv
        return parse_sdfv(b)


class GiVolume:
    """gi.rs:17-23 ambient-cube probe volume: cubes[(k*ny+j)*nx+i][face][rgb]."""

    def __init__(self, vmin, size, dims, cubes):
        self.min = _f3(vmin)
        self.size = _f3(size)
        self.dims = tuple(int(d) for d in dims)
        self.cubes = np.ascontiguousarray(cubes, dtype=F32).reshape(-1)


class Expr:
    """mm3e-kit/src/csg.rs:17-92 object-local CSG expression (tree)."""

    def __init__(self, kind, params=(), a=None, b=None, xform=None):
        self.kind = kind
        self.params = tuple(float(F32(p)) for p in params) + (0.0,) * (7 - len(params))
        self.a = a
        self.b = b
        self.xform = xform

    sphere = staticmethod(lambda r: Expr(abi.PRIM_SPHERE, (r,)))
    box = staticmethod(lambda half: Expr(abi.PRIM_BOX, tuple(half)))
    round_box = staticmethod(lambda half, radius: Expr(abi.PRIM_ROUND_BOX, tuple(half) + (radius,)))
    torus = staticmethod(lambda major, minor: Expr(abi.PRIM_TORUS, (major, minor)))
    cylinder = staticmethod(lambda h, r: Expr(abi.PRIM_CYLINDER, (h, r)))
    capsule = staticmethod(lambda a, b, r: Expr(abi.PRIM_CAPSULE, tuple(a) + tuple(b) + (r,)))
    cone = staticmethod(lambda r1, r2, h: Expr(abi.PRIM_CONE, (r1, r2, h)))
    ellipsoid = staticmethod(lambda r: Expr(abi.PRIM_ELLIPSOID, tuple(r)))
    octahedron = staticmethod(lambda s: Expr(abi.PRIM_OCTAHEDRON, (s,)))
    hex_prism = staticmethod(lambda r, h: Expr(abi.PRIM_HEX_PRISM, (r, h)))
    plane = staticmethod(lambda n, h: Expr(abi.PRIM_PLANE, tuple(n) + (h,)))
    transform = staticmethod(lambda shape, xform: Expr(abi.CSG_TRANSFORM, (), shape, None, xform))
    union = staticmethod(lambda a, b: Expr(abi.CSG_UNION, (), a, b))
    intersect = staticmethod(lambda a, b: Expr(abi.CSG_INTERSECT, (), a, b))
    subtract = staticmethod(lambda a, b: Expr(abi.CSG_SUBTRACT, (), a, b))
    smooth_union = staticmethod(lambda a, b, k: Expr(abi.CSG_SMOOTH_UNION, (k,), a, b))
    offset = staticmethod(lambda shape, d: Expr(abi.CSG_OFFSET, (d,), shape))
    shell = staticmethod(lambda shape, t: Expr(abi.CSG_SHELL, (t,), shape))

    def flatten(self, nodes):
        """Append this tree's nodes (children first) and return the root index."""
        ia = self.a.flatten(nodes) if self.a is not None else 0
        ib = self.b.flatten(nodes) if self.b is not None else 0
        n = abi.CsgNode()
        n.kind = self.kind
        n.a = ia
        n.b = ib
        n.params[:] = self.params
        xf = self.xform or Transform.IDENTITY
        n.rot[:] = xf.rot
        n.pos[:] = xf.pos
        n.scale = xf.scale
        nodes.append(n)
        return len(nodes) - 1


class DescHandle:
    """An `mm3e_scene_desc` plus the ctypes buffers it points into."""

    def __init__(self, desc, keep):
        self.desc = desc
        self._keep = keep

    @property
    def ptr(self):
        return C.byref(self.desc)


class Scene:
    """lib.rs:561-620 (defaults from Scene::new)."""

    def __init__(self, width, height):
        self.width = int(width)
        self.height = int(height)
        self.objects = []
        self.materials = [Material()]
        self.lights = []
        self.sun_dir = normalize_f32((0.6, 0.7, 0.4))
        self.ambient = _f3((0.02, 0.02, 0.02))
        self.sky_ambient = _f3((0.4, 0.4, 0.4))
        self.fog = _f3((0.62, 0.72, 0.86))
        self.fog_density = float(F32(0.012))
        self.aa = 2
        self.bounces = 1
        self.shadows = True
        self.ao = True
        self.marcher = Marcher()
        self.post = Post()
        self.mode = abi.MODE_BEAUTY
        self.gi = None
        self.volumes = []
        self.csgs = []

    def copy(self):
        s = _copy.copy(self)
        s.objects = list(self.objects)
        s.materials = list(self.materials)
        s.lights = list(self.lights)
        s.marcher = _copy.copy(self.marcher)
        s.post = _copy.copy(self.post)
        s.volumes = list(self.volumes)
        s.csgs = list(self.csgs)
        return s

    def material(self, m):
        self.materials.append(m)
        return len(self.materials) - 1

    def volume(self, v):
        """Scene::volume (lib.rs:631-638): raises normal_h to the volume's suggestion."""
        sug = v.recommended_normal_h()
        if math.isfinite(sug):
            self.marcher.normal_h = float(max(F32(self.marcher.normal_h), F32(sug)))
        self.volumes.append(v)
        return len(self.volumes) - 1

    def csg(self, expr):
        self.csgs.append(expr)
        return len(self.csgs) - 1

    def add(self, obj):
        self.objects.append(obj)

    def light(self, l):
        self.lights.append(l)

    def desc(self):
        keep = []
        d = abi.SceneDesc()
        d.width, d.height = self.width, self.height
        objs = (abi.Object * max(1, len(self.objects)))(*[o.to_abi() for o in self.objects])
        mats = (abi.Material * max(1, len(self.materials)))(*[m.to_abi() for m in self.materials])
        lts = (abi.Light * max(1, len(self.lights)))(*[l.to_abi() for l in self.lights])
        keep += [objs, mats, lts]
        d.objects, d.n_objects = objs, len(self.objects)
        d.materials, d.n_materials = mats, len(self.materials)
        d.lights, d.n_lights = lts, len(self.lights)
        d.sun_dir[:] = self.sun_dir
        d.ambient[:] = self.ambient
        d.sky_ambient[:] = self.sky_ambient
        d.fog[:] = self.fog
        d.fog_density = self.fog_density
        d.aa, d.bounces = int(self.aa), int(self.bounces)
        d.shadows, d.ao = int(bool(self.shadows)), int(bool(self.ao))
        d.marcher = self.marcher.to_abi()
        d.post = self.post.to_abi()
        d.mode = int(self.mode)
        if self.gi is not None:
            g = abi.Gi()
            g.min[:] = self.gi.min
            g.size[:] = self.gi.size
            g.nx, g.ny, g.nz = self.gi.dims
            g.cubes = self.gi.cubes.ctypes.data_as(C.POINTER(C.c_float))
            keep += [g, self.gi.cubes]
            d.gi = C.pointer(g)
        if self.volumes:
            vols = (abi.Volume * len(self.volumes))()
            for i, v in enumerate(self.volumes):
                vols[i].nx, vols[i].ny, vols[i].nz = v.dims
                vols[i].min[:] = v.min
                vols[i].cell[:] = v.cell
                vols[i].data = v.data.ctypes.data_as(C.POINTER(C.c_float))
                keep.append(v.data)
            keep.append(vols)
            d.volumes, d.n_volumes = vols, len(self.volumes)
        if self.csgs:
            nodes = []
            roots = [e.flatten(nodes) for e in self.csgs]
            arr = (abi.CsgNode * len(nodes))(*nodes)
            r = (C.c_uint32 * len(roots))(*roots)
            keep += [arr, r]
            d.csg_nodes, d.n_csg_nodes = arr, len(nodes)
            d.csg_roots, d.n_csgs = r, len(roots)
        return DescHandle(d, keep)


def look_at(eye, target, up_hint, fov_y):
    """Camera::look_at (camera.rs:50-55)."""
    cam = abi.Camera()
    _host_math.camera_look_at((C.c_float * 3)(*eye), (C.c_float * 3)(*target), (C.c_float * 3)(*up_hint), fov_y,
                              C.byref(cam))
    return cam


def orbit_camera(target, radius, yaw, pitch, fov_y):
    """orbit_camera (mm3e-orchestrator/src/lib.rs:1426-1435)."""
    cam = abi.Camera()
    _host_math.orbit_camera((C.c_float * 3)(*target), radius, yaw, pitch, fov_y, C.byref(cam))
    return cam


class DynSphere:
    """mm3e-cpu-parallel/src/lib.rs:18-23."""

    def __init__(self, pos, radius, albedo, metallic):
        self.pos, self.radius, self.albedo, self.metallic = _f3(pos), float(F32(radius)), _f3(albedo), float(
            F32(metallic))

    def to_abi(self):
        s = abi.DynSphere()
        s.pos[:] = self.pos
        s.radius = self.radius
        s.albedo[:] = self.albedo
        s.metallic = self.metallic
        return s
