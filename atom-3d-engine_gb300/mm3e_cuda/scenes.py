"""Seeded workload scenes: the benchmark configurations and the reference's own test scenes.

Every builder returns (Scene, camera) with fully specified parameters, so the GPU path, the
CPU oracle and the CPU baseline all render the identical description.

  spheres_scene     plain method, small: plane + three unit spheres, 960x540
  gallery_scene     feature gallery: the 11 primitives, smooth pair, domain ops, 1920x1080
  cornell_scene     Cornell-style GI room with a 32^3 ambient-cube probe volume, 1920x1080
  procedural_scene  seeded random scene (8-64 prims, CSG, domain ops) for the batched form
  demo_scene / canonical_scene / hero_scene  the reference's engine, backend and example scenes
"""
import math

import numpy as np

from . import abi
from .scene import (Expr, Light, Material, Object, Prim, Scene, SdfVolume, Transform, directional, look_at,
                    mat3_from_euler, orbit_camera, quat_to_mat3, radians)

F32 = np.float32


def spheres_scene(width=960, height=540, aa=1):
    """Plane y=0 (grey 0.8) + unit spheres at x = -2.2, 0, 2.2 (red/white/blue, roughness 0.5,
    metallic 0); one directional light (shadow k = 16 via angular radius 1/16) plus the constant
    and sky ambient of Scene::new; camera (0,2,-7) -> (0,1,0), 45 deg; max 128 steps, eps 1e-3,
    far 100, 64 shadow steps, 5 AO taps, no GI, no reflections."""
    s = Scene(width, height)
    s.aa = aa
    s.bounces = 0
    s.marcher.max_steps = 128
    s.marcher.eps = float(F32(1e-3))
    s.marcher.max_dist = 100.0
    s.marcher.shadow_steps = 64
    s.marcher.ao_samples = 5
    grey = s.material(Material.solid((0.8, 0.8, 0.8), roughness=0.5))
    red = s.material(Material.solid((0.85, 0.12, 0.10), roughness=0.5, metallic=0.0))
    white = s.material(Material.solid((0.9, 0.9, 0.9), roughness=0.5, metallic=0.0))
    blue = s.material(Material.solid((0.10, 0.20, 0.85), roughness=0.5, metallic=0.0))
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, grey))
    for x, m in ((-2.2, red), (0.0, white), (2.2, blue)):
        s.add(Object(Prim.sphere(1.0), Transform.at((x, 1.0, 0.0)), m))
    s.sun_dir = (0.0, 0.0, 0.0)
    sun = directional((0.45, 0.8, -0.4), (2.2, 2.1, 2.0)).soft(1.0 / 16.0)
    s.sun_dir = sun.vec
    s.light(sun)
    cam = look_at((0.0, 2.0, -7.0), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), radians(45.0))
    return s, cam


def gallery_scene(width=1920, height=1080, aa=1, seed=2):
    """4x3 grid of the 10 bounded analytic primitives plus a smooth-union pair (k = 0.3) and an
    emissive sphere, over a checker plane floor (the 11th primitive). Domain ops: twist 0.5
    rad/unit, bend, onion 0.05, round 0.1, repeat period 4, mirror. GGX materials with roughness
    uniform in [0.05, 1] and metallic in {0, 1} (seeded); soft shadows, AO, one reflection
    bounce, exponential fog, sky IBL, bloom and ACES; max 256 steps."""
    rng = np.random.default_rng(seed)
    s = Scene(width, height)
    s.aa = aa
    s.bounces = 1
    s.marcher.max_steps = 256
    s.marcher.step_scale = 0.6  # twist/bend are not distance preserving (gallery.rs:15)
    floor = s.material(Material.solid((1.0, 1.0, 1.0), checker=True, roughness=0.6, specular=0.2))

    def mat(albedo):
        rough = float(rng.uniform(0.05, 1.0))
        metal = float(rng.integers(0, 2))
        return s.material(Material.solid(albedo, roughness=rough, metallic=metal, specular=0.6,
                                         reflectivity=0.45 if metal > 0 else 0.0))

    palette = [(0.85, 0.25, 0.28), (0.95, 0.6, 0.2), (0.95, 0.82, 0.3), (0.35, 0.75, 0.4), (0.3, 0.6, 0.85),
               (0.55, 0.4, 0.8), (0.9, 0.5, 0.7), (0.8, 0.8, 0.8), (0.6, 0.35, 0.25), (0.25, 0.55, 0.55),
               (0.7, 0.7, 0.3), (0.5, 0.5, 0.9)]
    mats = [mat(c) for c in palette]
    glow = s.material(Material.solid((1.0, 0.9, 0.7), emissive=(6.0, 4.5, 2.5)))
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, floor))
    xs = [-4.5, -1.5, 1.5, 4.5]
    zs = [3.0, 0.0, -3.0]
    cells = [(x, z) for z in zs for x in xs]
    rot = lambda a, b, c: mat3_from_euler(a, b, c)
    # row 1
    s.add(Object(Prim.sphere(0.8), Transform.at((cells[0][0], 0.9, cells[0][1])), mats[0]).onion(0.05))
    s.add(Object(Prim.box((0.45, 1.1, 0.45)), Transform.at((cells[1][0], 1.1, cells[1][1])), mats[1]).twist(0.5))
    s.add(Object(Prim.round_box((0.7, 0.5, 0.6), 0.15), Transform.at((cells[2][0], 0.6, cells[2][1])).rotated(
        rot(0.0, 0.5, 0.0)), mats[2]))
    s.add(Object(Prim.torus(0.7, 0.25), Transform.at((cells[3][0], 1.0, cells[3][1])).rotated(rot(1.2, 0.0, 0.3)),
                 mats[3]))
    # row 2
    s.add(Object(Prim.cylinder(0.8, 0.5), Transform.at((cells[4][0], 0.8, cells[4][1])), mats[4]).round(0.1))
    s.add(Object(Prim.capsule((0.45, -0.5, 0.0), (0.45, 0.6, 0.0), 0.25), Transform.at((cells[5][0], 0.9,
                                                                                        cells[5][1])), mats[5])
          .mirror(True, False, False))
    s.add(Object(Prim.cone(0.7, 0.15, 1.3), Transform.at((cells[6][0], 0.7, cells[6][1])), mats[6]))
    s.add(Object(Prim.ellipsoid((0.5, 0.8, 0.6)), Transform.at((cells[7][0], 0.8, cells[7][1])), mats[7]))
    # row 3
    s.add(Object(Prim.octahedron(0.9), Transform.at((cells[8][0], 0.9, cells[8][1])).rotated(rot(0.0, 0.4, 0.0)),
                 mats[8]))
    s.add(Object(Prim.hex_prism(0.6, 0.5), Transform.at((cells[9][0], 0.6, cells[9][1])), mats[9]).bend(0.25))
    s.add(Object(Prim.sphere(0.65), Transform.at((cells[10][0] - 0.35, 0.75, cells[10][1])), mats[10]))
    s.add(Object(Prim.box((0.4, 0.4, 0.4)), Transform.at((cells[10][0] + 0.45, 0.55, cells[10][1])), mats[10])
          .smooth(0.3))
    s.add(Object(Prim.sphere(0.55), Transform.at((cells[11][0], 0.8, cells[11][1])), glow))
    # a repeated row of small lanterns behind the stage (period 4 along x)
    s.add(Object(Prim.octahedron(0.35), Transform.at((0.0, 2.6, -6.5)), mats[11]).repeat((4.0, 0.0, 0.0)))
    sun = directional((0.4, 0.8, 0.45), (2.6, 2.46, 2.16)).soft(0.04)
    s.sun_dir = sun.vec
    s.light(sun)
    s.light(Light.sphere((-3.0, 4.0, 3.0), (32.0, 34.0, 40.0), 1.0))
    cam = orbit_camera((0.0, 0.8, 0.0), 11.5, radians(100.0), 0.42, radians(52.0))
    return s, cam


def cornell_scene(width=1920, height=1080, aa=1, gi_dims=32):
    """Cornell-style room: five box walls (left red 0.63/0.06/0.05, right blue 0.05/0.06/0.63,
    the rest white 0.73), a white sphere r = 1 and a rotated 1x2x1 box, an emissive ceiling slab
    and a sphere light; soft shadows and AO. The GI probe volume (gi_dims^3 ambient cubes) is
    baked on the GPU from the same tape by the caller (CompiledScene.bake_gi)."""
    s = Scene(width, height)
    s.aa = aa
    s.bounces = 0
    s.fog_density = 0.0
    s.sky_ambient = (0.12, 0.12, 0.12)
    s.ambient = (0.0, 0.0, 0.0)
    white = s.material(Material.solid((0.73, 0.73, 0.73), roughness=0.8))
    red = s.material(Material.solid((0.63, 0.06, 0.05), roughness=0.8))
    blue = s.material(Material.solid((0.05, 0.06, 0.63), roughness=0.8))
    lamp = s.material(Material.solid((1.0, 1.0, 1.0), emissive=(4.0, 3.8, 3.4)))
    wall = lambda c, half, m: Object(Prim.box(half), Transform.at(c), m)
    s.add(wall((0.0, -0.1, 0.0), (3.0, 0.1, 3.0), white))   # floor
    s.add(wall((0.0, 6.1, 0.0), (3.0, 0.1, 3.0), white))    # ceiling
    s.add(wall((0.0, 3.0, -3.1), (3.0, 3.0, 0.1), white))   # back
    s.add(wall((-3.1, 3.0, 0.0), (0.1, 3.0, 3.0), red))     # left
    s.add(wall((3.1, 3.0, 0.0), (0.1, 3.0, 3.0), blue))     # right
    s.add(Object(Prim.sphere(1.0), Transform.at((-1.1, 1.0, 0.6)), white))
    s.add(Object(Prim.box((0.5, 1.0, 0.5)), Transform.at((1.2, 1.0, -0.8)).rotated(mat3_from_euler(0.0, 0.45, 0.0)),
                 white))
    s.add(Object(Prim.box((1.0, 0.05, 1.0)), Transform.at((0.0, 5.95, 0.0)), lamp))
    s.sun_dir = (0.0, 1.0, 0.0)
    s.light(Light.sphere((0.0, 5.4, 0.0), (16.0, 15.5, 14.5), 0.8))
    cam = look_at((0.0, 3.0, 9.5), (0.0, 2.8, 0.0), (0.0, 1.0, 0.0), radians(45.0))
    return s, cam


def _random_prim(rng):
    kind = int(rng.integers(0, 11))
    u = lambda: float(rng.uniform(0.2, 1.5))
    if kind == 0:
        return Prim.sphere(u())
    if kind == 1:
        return Prim.box((u(), u(), u()))
    if kind == 2:
        h = (u(), u(), u())
        return Prim.round_box(h, 0.3 * min(h))
    if kind == 3:
        a = u()
        return Prim.torus(a, min(a, u()) * 0.4)
    if kind == 4:
        return Prim.cylinder(u(), u())
    if kind == 5:
        return Prim.capsule((0.0, -u() * 0.5, 0.0), (0.0, u() * 0.5, 0.0), u() * 0.5)
    if kind == 6:
        h = u() + 0.5
        return Prim.cone(min(u(), h * 0.9), min(u() * 0.3, h * 0.9), h)
    if kind == 7:
        return Prim.ellipsoid((u(), u(), u()))
    if kind == 8:
        return Prim.octahedron(u())
    if kind == 9:
        return Prim.hex_prism(u(), u())
    return Prim.plane((0.0, 1.0, 0.0), 5.0)


def _random_expr(rng, depth):
    """Object-local CSG tree (csg::Expr) of the given depth: intersect lives here only."""
    if depth <= 0 or rng.random() < 0.3:
        p = _random_prim(rng)
        while p.kind == abi.PRIM_PLANE:
            p = _random_prim(rng)
        prim = Expr(p.kind, p.params[:7])
        if rng.random() < 0.5:
            q = rng.normal(size=4)
            q /= np.linalg.norm(q)
            return Expr.transform(prim, Transform.at(tuple(rng.uniform(-0.5, 0.5, 3))).rotated(quat_to_mat3(tuple(q))))
        return prim
    a = _random_expr(rng, depth - 1)
    b = _random_expr(rng, depth - 1)
    r = rng.random()
    if r < 0.4:
        return Expr.union(a, b)
    if r < 0.6:
        return Expr.intersect(a, b)
    if r < 0.8:
        return Expr.subtract(a, b)
    return Expr.smooth_union(a, b, float(rng.uniform(0.05, 0.4)))


def procedural_scene(seed, width=None, height=None, max_depth=4):
    """Seeded random scene: 8-64 primitives, types uniform over the 11, positions U[-5,5]^3,
    sizes U[0.2,1.5], random unit-quaternion rotations; scene-level combine is union / smooth /
    subtract (p = 0.6/0.2/0.2 with intersect, which a scene-level Combine cannot express, folded
    into object-local CSG trees of depth <= max_depth); 0-2 domain ops per object; resolution
    uniform over {256^2, 512^2, 1280x720, 1920x1080}; orbit camera; config-1 shading set."""
    rng = np.random.default_rng(seed)
    res = [(256, 256), (512, 512), (1280, 720), (1920, 1080)][int(rng.integers(0, 4))]
    w, h = (width, height) if width else res
    s = Scene(w, h)
    s.aa = 1
    s.bounces = 0
    s.marcher.max_steps = 128
    s.marcher.eps = float(F32(1e-3))
    s.marcher.max_dist = 100.0
    s.marcher.step_scale = 0.7
    n = int(rng.integers(8, 65))
    for i in range(6):
        s.material(Material.solid(tuple(rng.uniform(0.1, 0.95, 3)), roughness=float(rng.uniform(0.1, 0.9)),
                                  metallic=float(rng.integers(0, 2))))
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 6.0), Transform.IDENTITY, 1))
    for i in range(n):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        pos = tuple(rng.uniform(-5.0, 5.0, 3))
        if rng.random() < 0.15:
            eid = s.csg(_random_expr(rng, max_depth - 1))
            prim = Prim.csg(eid)
        else:
            prim = _random_prim(rng)
            if prim.kind == abi.PRIM_PLANE:
                prim = Prim.sphere(float(rng.uniform(0.2, 1.5)))
        o = Object(prim, Transform.at(pos).rotated(quat_to_mat3(tuple(q))), int(rng.integers(1, 7)))
        r = rng.random()
        if r < 0.2:
            o = o.smooth(float(rng.uniform(0.1, 0.5)))
        elif r < 0.4:
            o = o.subtract()
        for _ in range(int(rng.integers(0, 3))):
            op = int(rng.integers(0, 6))
            if op == 0:
                o = o.twist(float(rng.uniform(-0.6, 0.6)))
            elif op == 1:
                o = o.bend(float(rng.uniform(-0.4, 0.4)))
            elif op == 2:
                o = o.onion(float(rng.uniform(0.03, 0.1)))
            elif op == 3:
                o = o.round(float(rng.uniform(0.02, 0.15)))
            elif op == 4:
                o = o.mirror(bool(rng.integers(0, 2)), bool(rng.integers(0, 2)), bool(rng.integers(0, 2)))
            else:
                o = o.elongate(tuple(rng.uniform(0.0, 0.5, 3)))
        s.add(o)
    sun = directional((0.5, 0.8, 0.3), (2.0, 1.95, 1.85)).soft(1.0 / 16.0)
    s.sun_dir = sun.vec
    s.light(sun)
    cam = orbit_camera((0.0, 0.0, 0.0), float(rng.uniform(12.0, 16.0)), float(rng.uniform(-math.pi, math.pi)),
                       float(rng.uniform(0.1, 0.7)), radians(50.0))
    return s, cam


# ---- the reference's own scenes ------------------------------------------------------------

def hero_scene(width=960, height=540, aa=2, bounces=2):
    """mm3e-orchestrator/examples/spheres.rs:11-63 and cpu_bench.rs:72-108 (the published-fps scene)."""
    s = Scene(width, height)
    s.aa = aa
    s.bounces = bounces
    floor = s.material(Material.solid((1.0, 1.0, 1.0), checker=True, specular=0.15, roughness=0.6))
    red = s.material(Material.solid((0.85, 0.18, 0.20), specular=0.7, roughness=0.25))
    gold = s.material(Material.solid((0.95, 0.72, 0.25), metallic=1.0, roughness=0.18, reflectivity=0.5))
    glassy = s.material(Material.solid((0.20, 0.55, 0.85), specular=0.9, roughness=0.15, reflectivity=0.35))
    mirror = s.material(Material.solid((0.95, 0.95, 0.95), metallic=1.0, roughness=0.05, reflectivity=0.85))
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, floor))
    s.add(Object(Prim.sphere(1.0), Transform.at((-2.4, 1.0, 0.2)), mirror))
    s.add(Object(Prim.round_box((0.85, 0.85, 0.85), 0.18), Transform.at((0.2, 0.95, -0.6)).rotated(
        mat3_from_euler(0.0, 0.6, 0.0)), gold))
    s.add(Object(Prim.torus(0.85, 0.30), Transform.at((2.6, 1.05, 0.4)).rotated(mat3_from_euler(1.2, 0.0, 0.2)),
                 glassy))
    s.add(Object(Prim.sphere(0.7), Transform.at((0.9, 0.7, 1.9)), red))
    s.add(Object(Prim.capsule((0.0, -0.5, 0.0), (0.0, 0.6, 0.0), 0.4), Transform.at((1.55, 0.7, 1.9)), red)
          .smooth(0.5))
    sun = directional((0.55, 0.7, 0.35), tuple(float(F32(c) * F32(1.6)) for c in (1.25, 1.12, 0.95)))
    s.sun_dir = sun.vec
    s.light(sun)
    s.light(directional((-0.4, 0.5, -0.7), (0.35, 0.42, 0.6)))
    cam = orbit_camera((0.2, 0.85, 0.4), 8.5, 0.55, 0.32, radians(50.0))
    return s, cam


def gpu_render_scene(width=960, height=540, yaw=0.55):
    """mm3e-gpu/examples/gpu_render.rs:11-49 (and gpu_resolution.rs): the hero scene at aa 2 with 3
    bounces and a soft sun (radius 0.04), the scene of the reference's published GPU frame rates;
    orbit camera at `yaw` (the benchmark loop turns it by 0.01 per frame from 0.55)."""
    s, _ = hero_scene(width, height, 2, 3)
    s.lights[0] = s.lights[0].soft(0.04)
    cam = orbit_camera((0.2, 0.85, 0.4), 8.5, yaw, 0.32, radians(50.0))
    return s, cam


def demo_scene():
    """mm3e-orchestrator/tests/engine.rs:11-27 with its camera (engine.rs:29-31)."""
    s = Scene(96, 64)
    s.aa = 1
    floor = s.material(Material.solid((1.0, 1.0, 1.0), checker=True, roughness=0.6))
    red = s.material(Material.solid((0.85, 0.2, 0.2), roughness=0.3))
    metal = s.material(Material.solid((0.9, 0.8, 0.4), metallic=1.0, roughness=0.2, reflectivity=0.4))
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, floor))
    s.add(Object(Prim.sphere(1.0), Transform.at((-1.2, 1.0, 0.0)), red).round(0.1))
    s.add(Object(Prim.torus(0.7, 0.25), Transform.at((1.2, 1.0, 0.0)), metal))
    s.add(Object(Prim.box((0.6, 0.6, 0.6)), Transform.at((0.0, 0.6, 1.6)), red).onion(0.05))
    sun = directional((0.5, 0.75, 0.4), (2.0, 2.0, 2.0)).soft(0.04)
    s.sun_dir = sun.vec
    s.light(sun)
    s.light(Light.sphere((-3.0, 4.0, 3.0), (20.0, 20.0, 20.0), 1.0))
    cam = orbit_camera((0.0, 0.8, 0.3), 7.0, 0.5, 0.3, radians(52.0))
    return s, cam


def canonical_scene():
    """mm3e-cpu-parallel/tests/canonical.rs:15-29: 65x41, aa 1, no bounces/ambient/fog/AO/
    shadows/bloom, camera (0,0,5) -> origin, 45 deg."""
    s = Scene(65, 41)
    s.aa = 1
    s.bounces = 0
    s.ambient = (0.0, 0.0, 0.0)
    s.sky_ambient = (0.0, 0.0, 0.0)
    s.fog_density = 0.0
    s.ao = False
    s.shadows = False
    s.post.bloom = False
    cam = look_at((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), radians(45.0))
    return s, cam


def canonical_asset_scene():
    """canonical.rs:119-149: a sampled SDF volume, an object-local CSG subtraction and a
    constant 2x2x2 GI volume."""
    from .scene import GiVolume
    s, cam = canonical_scene()
    red = s.material(Material.solid((0.8, 0.05, 0.05)))
    blue = s.material(Material.solid((0.05, 0.08, 0.8)))
    dims = 9
    low = F32(-1.25)
    cell = F32(F32(2.5) / F32(dims - 1))
    samples = []
    for z in range(dims):
        for y in range(dims):
            for x in range(dims):
                p = np.array([low + F32(x) * cell, low + F32(y) * cell, low + F32(z) * cell], dtype=F32)
                ln = np.sqrt(F32(F32(p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]), dtype=F32)
                samples.append(F32(ln - F32(0.8)))
    vid = s.volume(SdfVolume((dims, dims, dims), (low, low, low), (cell, cell, cell), np.array(samples, F32)))
    s.add(Object(Prim.volume(vid), Transform.at((-1.25, 0.0, 0.0)), red))
    eid = s.csg(Expr.subtract(Expr.sphere(0.85), Expr.capsule((0.0, 0.0, -1.2), (0.0, 0.0, 1.2), 0.3)))
    s.add(Object(Prim.csg(eid), Transform.at((1.25, 0.0, 0.0)), blue))
    cubes = np.tile(np.array([0.1, 0.3, 0.1], F32), 8 * 6)
    s.gi = GiVolume((-3.0, -3.0, -3.0), (6.0, 6.0, 6.0), (2, 2, 2), cubes)
    s.post.exposure = float(F32(1.2))
    return s, cam


def reference_gallery_scene():
    """mm3e-orchestrator/examples/gallery.rs:11-84 (1100x560, aa 2, 2 bounces)."""
    s = Scene(1100, 560)
    s.aa = 2
    s.bounces = 2
    s.marcher.step_scale = 0.6
    s.fog_density = 0.01
    floor = s.material(Material.solid((1.0, 1.0, 1.0), checker=True, roughness=0.6, specular=0.2))
    palette = []
    for c in [(0.85, 0.25, 0.28), (0.95, 0.6, 0.2), (0.95, 0.82, 0.3), (0.35, 0.75, 0.4), (0.3, 0.6, 0.85),
              (0.55, 0.4, 0.8), (0.9, 0.5, 0.7)]:
        palette.append(s.material(Material.solid(c, roughness=0.3, specular=0.7)))
    gold = s.material(Material.solid((0.95, 0.72, 0.28), metallic=1.0, roughness=0.2, reflectivity=0.5))
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, floor))
    prims = [Prim.sphere(0.6), Prim.box((0.55, 0.55, 0.55)), Prim.torus(0.5, 0.2), Prim.cone(0.6, 0.05, 1.1),
             Prim.ellipsoid((0.4, 0.65, 0.5)), Prim.octahedron(0.8), Prim.hex_prism(0.55, 0.5)]
    for i, p in enumerate(prims):
        x = float(F32(-3.6) + F32(i) * F32(1.2))
        s.add(Object(p, Transform.at((x, 0.7, 1.6)), palette[i]))
    s.add(Object(Prim.box((0.45, 1.3, 0.45)), Transform.at((-2.6, 1.3, -1.4)), gold).twist(0.9))
    s.add(Object(Prim.sphere(0.9), Transform.at((-0.6, 1.0, -1.4)), palette[4]).onion(0.06))
    s.add(Object(Prim.box((0.8, 0.8, 0.8)), Transform.at((1.4, 0.95, -1.4)), palette[1]).round(0.35))
    s.add(Object(Prim.sphere(0.7), Transform.at((3.2, 0.9, -1.4)), palette[3]))
    s.add(Object(Prim.capsule((0.0, -0.6, 0.0), (0.0, 0.7, 0.0), 0.35), Transform.at((3.7, 0.9, -1.4)).rotated(
        mat3_from_euler(0.0, 0.0, 0.5)), palette[3]).smooth(0.5))
    sun = directional((0.4, 0.8, 0.45), tuple(float(F32(c) * F32(2.2)) for c in (1.2, 1.12, 0.98))).soft(0.04)
    s.sun_dir = sun.vec
    s.light(sun)
    s.light(Light.sphere((-3.0, 4.0, 3.0), tuple(float(F32(c) * F32(40.0)) for c in (0.8, 0.85, 1.0)), 1.0))
    cam = orbit_camera((0.0, 0.75, 0.2), 8.6, 0.58, 0.40, radians(52.0))
    return s, cam


def reference_gi_demo_scene():
    """mm3e-orchestrator/examples/gi_demo.rs:11-58 (800x600, aa 3, 1 bounce); the caller bakes
    GI with dims (20, 14, 20) and 5 samples, as the example does."""
    s = Scene(800, 600)
    s.aa = 3
    s.bounces = 1
    s.fog_density = 0.0
    s.sky_ambient = (0.18, 0.18, 0.18)
    s.ambient = (0.0, 0.0, 0.0)
    white = s.material(Material.solid((0.85, 0.85, 0.85), roughness=0.7))
    red = s.material(Material.solid((0.85, 0.12, 0.12), roughness=0.7))
    blue = s.material(Material.solid((0.12, 0.2, 0.85), roughness=0.7))
    chrome = s.material(Material.solid((0.9, 0.9, 0.9), metallic=1.0, roughness=0.12, reflectivity=0.7))
    wall = lambda c, half, m: Object(Prim.box(half), Transform.at(c), m)
    s.add(wall((0.0, -0.1, 0.0), (4.0, 0.1, 4.0), white))
    s.add(wall((0.0, 4.1, 0.0), (4.0, 0.1, 4.0), white))
    s.add(wall((0.0, 2.0, -4.1), (4.0, 4.0, 0.1), white))
    s.add(wall((-4.1, 2.0, 0.0), (0.1, 4.0, 4.0), red))
    s.add(wall((4.1, 2.0, 0.0), (0.1, 4.0, 4.0), blue))
    s.add(Object(Prim.sphere(1.1), Transform.at((-1.3, 1.1, 0.4)), white))
    s.add(Object(Prim.sphere(1.0), Transform.at((1.5, 1.0, -0.6)), chrome))
    lamp = s.material(Material.solid((1.0, 1.0, 1.0), emissive=(3.0, 3.0, 3.0)))
    s.add(Object(Prim.box((1.4, 0.06, 1.4)), Transform.at((0.0, 3.9, 0.0)), lamp))
    from .scene import normalize_f32
    s.sun_dir = normalize_f32((0.0, 1.0, 0.2))
    s.light(Light.sphere((0.0, 3.7, 0.0), (14.0, 14.0, 14.0), 1.2))
    cam = look_at((0.0, 2.0, 7.5), (0.0, 1.6, 0.0), (0.0, 1.0, 0.0), radians(50.0))
    return s, cam


# ------------------------------------------------------------------------------------------
# Meshes for the mesh -> SDF bake (the served stream's mesh requests). The reference has no
# icosphere or noise generator; these are seeded generators of this package.
# ------------------------------------------------------------------------------------------
def uv_sphere_mesh(rings, segments, radius):
    """UV sphere with poles, as the reference's engine tests build it (tests/engine.rs:370-401):
    (positions (n, 3) f32, triangles (m, 3) u32)."""
    pos = [(0.0, radius, 0.0)]
    for r in range(1, rings):
        phi = np.float32(math.pi) * np.float32(r) / np.float32(rings)
        for s in range(segments):
            theta = np.float32(2.0 * math.pi) * np.float32(s) / np.float32(segments)
            pos.append((radius * np.sin(phi) * np.cos(theta), radius * np.cos(phi), radius * np.sin(phi) * np.sin(theta)))
    pos.append((0.0, -radius, 0.0))

    def ring(r, s):
        return 1 + (r - 1) * segments + (s % segments)

    tris = [(0, ring(1, s + 1), ring(1, s)) for s in range(segments)]
    for r in range(1, rings - 1):
        for s in range(segments):
            a, b, c, d = ring(r, s), ring(r, s + 1), ring(r + 1, s + 1), ring(r + 1, s)
            tris += [(a, b, c), (a, c, d)]
    south = len(pos) - 1
    tris += [(south, ring(rings - 1, s), ring(rings - 1, s + 1)) for s in range(segments)]
    return np.asarray(pos, np.float32), np.asarray(tris, np.uint32)


def icosphere(subdivisions):
    """Unit icosphere: the icosahedron with every triangle split into four `subdivisions` times,
    new vertices projected to the sphere. 10*4^n + 2 vertices, 20*4^n triangles."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [tuple(np.asarray(v, np.float64) / np.linalg.norm(v)) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = (np.asarray(verts[a]) + np.asarray(verts[b])) * 0.5
                verts.append(tuple(m / np.linalg.norm(m)))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.asarray(verts, np.float64), np.asarray(faces, np.uint32)


def value_noise3(p, seed):
    """Seeded 3-D value noise in [-1, 1]: hashed lattice values, smoothstep-weighted trilinear
    blend. p: (n, 3) float64."""
    p = np.asarray(p, np.float64)
    i0 = np.floor(p).astype(np.int64)
    f = p - i0
    w = f * f * (3.0 - 2.0 * f)

    def lattice(ix, iy, iz):
        h = (ix * 73856093) ^ (iy * 19349663) ^ (iz * 83492791) ^ (seed * 2654435761)
        h = (h ^ (h >> 13)) * 1274126177
        h = h ^ (h >> 16)
        return (h & 0xFFFF).astype(np.float64) / 32767.5 - 1.0

    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out = out + wx * wy * wz * lattice(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
    return out


def displaced_icosphere(seed, subdivisions=5, amplitude=0.15, octaves=3, frequency=2.0, radius=1.0):
    """Icosphere (subdivision 5: 20,480 triangles) displaced radially by `octaves`-octave value
    noise of amplitude `amplitude`: (positions f32 (n, 3), triangles u32 (m, 3))."""
    v, f = icosphere(subdivisions)
    n = np.zeros(len(v))
    amp, freq, norm = 1.0, frequency, 0.0
    for o in range(octaves):
        n += amp * value_noise3(v * freq, seed * 131 + o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    r = radius * (1.0 + amplitude * n / norm)
    return (v * r[:, None]).astype(np.float32), f


def mesh_volume_scene(volume, seed=0, width=512, height=512):
    """A served-stream scene around a baked mesh volume: the volume object on a ground plane,
    config-1 shading, orbit camera."""
    rng = np.random.default_rng(seed)
    s = Scene(width, height)
    s.aa = 1
    s.bounces = 0
    s.marcher.max_steps = 128
    s.marcher.eps = float(F32(1e-3))
    s.marcher.max_dist = 100.0
    s.marcher.normal_h = volume.recommended_normal_h()
    grey = s.material(Material.solid((0.8, 0.8, 0.8)))
    mat = s.material(Material.solid(tuple(rng.uniform(0.2, 0.9, 3)), roughness=0.5))
    vid = s.volume(volume)
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, grey))
    s.add(Object(Prim.volume(vid), Transform.at((0.0, 1.2, 0.0)), mat))
    s.light(directional((0.4, 0.8, -0.45), (1.0, 1.0, 1.0)).soft(1.0 / 16.0))
    s.ambient = (0.08, 0.08, 0.1)
    cam = orbit_camera((0.0, 1.0, 0.0), 4.5, float(rng.uniform(-math.pi, math.pi)), 0.35, math.radians(45.0))
    return s, cam
