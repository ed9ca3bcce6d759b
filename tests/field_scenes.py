"""Seeded test scenes for the world-field paths (shared by the GPU parity and specialisation tests)."""
import numpy as np

from mm3e_cuda.scene import Material, Object, Prim, Scene, Transform, look_at, mat3_from_euler, radians


def noncons_scene(seed, width=64, height=36):
    """A union run dominated by ellipsoids and octahedra (fields that can undercut their bounding
    spheres) among spheres and boxes, on a plane; with a camera looking at it."""
    rng = np.random.default_rng(seed)
    s = Scene(width, height)
    s.materials = [Material((0.8, 0.8, 0.8)), Material((0.7, 0.2, 0.2)), Material((0.2, 0.6, 0.3))]
    s.objects = [Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, 0)]
    for k in range(18):
        pos = tuple(float(v) for v in rng.uniform([-4, 0.3, -4], [4, 2.5, 4]))
        rot = mat3_from_euler(*rng.uniform(-1.5, 1.5, 3))
        kind = k % 4
        if kind == 0:
            prim = Prim.octahedron(float(rng.uniform(0.3, 1.0)))
        elif kind == 1:
            prim = Prim.ellipsoid(tuple(float(v) for v in rng.uniform(0.2, 1.0, 3)))
        elif kind == 2:
            prim = Prim.sphere(float(rng.uniform(0.2, 0.8)))
        else:
            prim = Prim.box(tuple(float(v) for v in rng.uniform(0.2, 0.7, 3)))
        s.objects.append(Object(prim, Transform(pos, rot, float(rng.uniform(0.7, 1.3))), 1 + k % 2))
    cam = look_at((0.0, 3.5, -9.0), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), radians(50.0))
    return s, cam
