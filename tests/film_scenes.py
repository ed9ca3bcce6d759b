"""Scenes of the reference's render_film tests (mm3e-orchestrator/tests/film.rs:5-27), shared by
the CPU (oracle) and GPU film tests."""
import numpy as np

from mm3e_cuda.scene import Light, Material, Object, Prim, Scene, Transform, directional, look_at


def camera():
    return look_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 0.8)


def emissive_scene(width, height, emission):
    s = Scene(width, height)
    s.aa = 4
    s.ao = False
    s.shadows = False
    s.bounces = 0
    s.fog_density = 0.0
    s.ambient = (0.0, 0.0, 0.0)
    s.sky_ambient = (0.0, 0.0, 0.0)
    s.marcher.eps = float(np.float32(0.00001))
    s.marcher.max_steps = 512
    m = s.material(Material(albedo=(0.0, 0.0, 0.0), emissive=emission))
    s.add(Object(Prim.sphere(0.55), Transform.IDENTITY, m))
    return s


def reflective_scene():
    """film.rs:29-42: aa 3, two bounces, a reflective sphere and a directional light."""
    s = Scene(23, 19)
    s.aa = 3
    s.bounces = 2
    m = s.material(Material(albedo=(0.9, 0.1, 0.06), reflectivity=0.7))
    s.add(Object(Prim.sphere(0.65), Transform.IDENTITY, m))
    s.light(directional((-1.0, 2.0, 2.0), (3.0, 3.0, 3.0)))
    return s
