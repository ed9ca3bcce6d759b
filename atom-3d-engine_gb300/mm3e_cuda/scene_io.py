"""`.mm3e` text scenes (mm3e-orchestrator/src/scene_io.rs) and `.sdfv` volumes
(mm3e-kit/src/volume.rs:115-187) through the library's parsers and writers."""
import ctypes as C

import numpy as np

from . import abi
from .native import lib
from .scene import Light, Material, Object, Prim, Scene, SdfVolume, Transform


class SceneFormatError(ValueError):
    pass


def _scene_from_desc(d):
    s = Scene(d.width, d.height)
    s.objects, s.materials, s.lights = [], [], []
    for i in range(d.n_materials):
        m = d.materials[i]
        s.materials.append(Material(tuple(m.albedo), m.metallic, m.specular, m.roughness, m.reflectivity,
                                    tuple(m.emissive), bool(m.checker)))
    for i in range(d.n_lights):
        l = d.lights[i]
        s.lights.append(Light(tuple(l.vec), tuple(l.color), bool(l.directional), l.radius))
    for i in range(d.n_objects):
        o = d.objects[i]
        obj = Object(Prim(o.prim, tuple(o.params), o.id), Transform(tuple(o.pos), tuple(o.rot), o.scale), o.mat)
        obj.combine, obj.k = o.combine, o.smooth_k
        obj.mirror_ = (bool(o.mirror & 1), bool(o.mirror & 2), bool(o.mirror & 4))
        obj.repeat_, obj.elongate_ = tuple(o.repeat), tuple(o.elongate)
        obj.twist_, obj.bend_, obj.round_, obj.onion_ = o.twist, o.bend, o.round, o.onion
        s.objects.append(obj)
    s.sun_dir, s.ambient, s.sky_ambient, s.fog = (tuple(d.sun_dir), tuple(d.ambient), tuple(d.sky_ambient),
                                                   tuple(d.fog))
    s.fog_density, s.aa, s.bounces = d.fog_density, d.aa, d.bounces
    s.shadows, s.ao, s.mode = bool(d.shadows), bool(d.ao), d.mode
    for k in ("max_steps", "max_dist", "eps", "step_scale", "shadow_steps", "ao_samples", "lod_footprint",
              "subitize", "normal_h"):
        setattr(s.marcher, k, getattr(d.marcher, k))
    s.marcher.secant = bool(d.marcher.secant)
    for k in ("exposure", "bloom_threshold", "bloom_intensity", "bloom_radius"):
        setattr(s.post, k, getattr(d.post, k))
    s.post.bloom = bool(d.post.bloom)
    return s


def parse(text):
    """scene_io::parse: (Scene, Camera). Raises SceneFormatError with the reference's message."""
    err = C.create_string_buffer(512)
    ptr = C.c_void_p()
    rc = lib().mm3e_scene_parse_mm3e(text.encode(), C.byref(ptr), err, 512)
    if rc != abi.OK:
        raise SceneFormatError(err.value.decode(errors="replace"))
    try:
        scene = _scene_from_desc(lib().mm3e_parsed_scene_desc(ptr).contents)
        cam = abi.Camera()
        lib().mm3e_parsed_scene_camera(ptr, C.byref(cam))
    finally:
        lib().mm3e_parsed_scene_free(ptr)
    return scene, cam


def serialize(scene, camera):
    """scene_io::try_serialize: the `.mm3e` text."""
    h = scene.desc()
    n = C.c_size_t()
    err = C.create_string_buffer(512)
    rc = lib().mm3e_scene_write_mm3e(h.ptr, C.byref(camera), None, 0, C.byref(n), err, 512)
    if rc != abi.OK:
        raise SceneFormatError(err.value.decode(errors="replace"))
    buf = C.create_string_buffer(n.value + 1)
    lib().mm3e_scene_write_mm3e(h.ptr, C.byref(camera), buf, n.value + 1, C.byref(n), err, 512)
    return buf.value.decode()


def parse_sdfv(data):
    """SdfVolume::from_sdfv_bytes: an SdfVolume. Raises SceneFormatError with the reference's message."""
    b = np.frombuffer(bytes(data), np.uint8)
    P = C.POINTER
    ptr = b.ctypes.data_as(P(C.c_uint8))
    v = abi.Volume()
    n = C.c_size_t()
    err = C.create_string_buffer(512)
    rc = lib().mm3e_volume_parse_sdfv(ptr, len(b), C.byref(v), None, 0, C.byref(n), err, 512)
    if rc != abi.OK:
        raise SceneFormatError(err.value.decode(errors="replace"))
    out = np.empty(n.value, np.float32)
    rc = lib().mm3e_volume_parse_sdfv(ptr, len(b), C.byref(v), out.ctypes.data_as(P(C.c_float)), n.value, None,
                                      err, 512)
    if rc != abi.OK:
        raise SceneFormatError(err.value.decode(errors="replace"))
    return SdfVolume((v.nx, v.ny, v.nz), tuple(v.min), tuple(v.cell), out)


def serialize_sdfv(vol):
    """SdfVolume::to_sdfv_bytes: the `.sdfv` bytes."""
    data = np.ascontiguousarray(vol.data, np.float32)
    v = abi.Volume()
    v.nx, v.ny, v.nz = (int(d) for d in vol.dims)
    v.min[:] = [float(x) for x in vol.min]
    v.cell[:] = [float(x) for x in vol.cell]
    v.data = data.ctypes.data_as(C.POINTER(C.c_float))
    n = C.c_size_t()
    err = C.create_string_buffer(512)
    rc = lib().mm3e_volume_write_sdfv(C.byref(v), None, 0, C.byref(n), err, 512)
    if rc != abi.OK:
        raise SceneFormatError(err.value.decode(errors="replace"))
    out = (C.c_uint8 * n.value)()
    rc = lib().mm3e_volume_write_sdfv(C.byref(v), out, n.value, C.byref(n), err, 512)
    if rc != abi.OK:
        raise SceneFormatError(err.value.decode(errors="replace"))
    return bytes(out)
