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


def smooth_chain_scene(seed, width=64, height=36):
    """Plain-union runs interleaved with smooth-union objects of blend radii from 0 to 1.2 and a
    subtraction, identity and rotated transforms mixed, on a plane: the specialised field's
    segment skip (a far smooth-union object leaves the accumulator as it is) meets accumulators of
    both signs, including points inside the union (AO and normal taps)."""
    rng = np.random.default_rng(seed)
    s = Scene(width, height)
    s.materials = [Material((0.8, 0.8, 0.8)), Material((0.7, 0.3, 0.2)), Material((0.2, 0.5, 0.7))]
    s.objects = [Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, 0)]
    ks = [0.0, 0.05, 0.3, 0.7, 1.2]
    for k in range(16):
        pos = tuple(float(v) for v in rng.uniform([-4, 0.3, -3], [4, 2.0, 3]))
        rot = mat3_from_euler(*rng.uniform(-1.2, 1.2, 3)) if k % 3 else (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)
        prim = Prim.sphere(float(rng.uniform(0.3, 0.9))) if k % 2 else Prim.box(tuple(float(v) for v in rng.uniform(0.2, 0.7, 3)))
        o = Object(prim, Transform(pos, rot, 1.0), 1 + k % 2)
        if k % 4 == 1:
            o = o.smooth(ks[(k // 4) % len(ks)])
        elif k == 10:
            o = o.subtract()
        elif k % 4 == 3:
            o = o.smooth(ks[(k // 4 + 2) % len(ks)])
        s.objects.append(o)
    cam = look_at((0.5, 3.0, -8.5), (0.0, 0.8, 0.0), (0.0, 1.0, 0.0), radians(55.0))
    return s, cam


def csg_zoo_scene(seed, width=64, height=36):
    """Objects whose shapes are CSG programs over every operation (union, intersection,
    subtraction, smooth union, offset, shell, nested transforms with rotations and scales), some of
    the objects also rounded, onioned, mirrored or smooth-unioned, on a plane; with a camera
    looking at them."""
    from mm3e_cuda import abi
    from mm3e_cuda.scene import Expr
    from mm3e_cuda.scenes import _random_prim

    rng = np.random.default_rng(seed)
    s = Scene(width, height)
    s.materials = [Material((0.8, 0.8, 0.8)), Material((0.7, 0.25, 0.2)), Material((0.2, 0.5, 0.7))]
    s.objects = [Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, 0)]

    def leaf():
        p = _random_prim(rng)
        while p.kind == abi.PRIM_PLANE:
            p = _random_prim(rng)
        e = Expr(p.kind, tuple(float(v) * 0.6 for v in p.params[:7]) if p.kind != abi.PRIM_CAPSULE else p.params[:7])
        return e

    def tree(depth):
        if depth == 0:
            return leaf()
        op = int(rng.integers(0, 7))
        if op == 0:
            return Expr.union(tree(depth - 1), tree(depth - 1))
        if op == 1:
            return Expr.intersect(tree(depth - 1), leaf())
        if op == 2:
            return Expr.subtract(tree(depth - 1), tree(depth - 1))
        if op == 3:
            return Expr.smooth_union(tree(depth - 1), tree(depth - 1), float(rng.uniform(0.05, 0.4)))
        if op == 4:
            return Expr.offset(tree(depth - 1), float(rng.uniform(-0.05, 0.1)))
        if op == 5:
            return Expr.shell(tree(depth - 1), float(rng.uniform(0.02, 0.08)))
        rot = mat3_from_euler(*rng.uniform(-1.5, 1.5, 3))
        return Expr.transform(tree(depth - 1), Transform(tuple(rng.uniform(-0.4, 0.4, 3)), rot,
                                                         float(rng.uniform(0.6, 1.4))))

    for k in range(10):
        pos = tuple(float(v) for v in rng.uniform([-4, 0.6, -3], [4, 2.2, 3]))
        rot = mat3_from_euler(*rng.uniform(-1.2, 1.2, 3))
        o = Object(Prim.csg(s.csg(tree(int(rng.integers(1, 4))))), Transform(pos, rot, float(rng.uniform(0.7, 1.3))),
                   1 + k % 2)
        if k % 5 == 1:
            o = o.round(0.05)
        elif k % 5 == 2:
            o = o.onion(0.04)
        elif k % 5 == 3:
            o = o.mirror(True, False, bool(k % 2))
        if k == 4:
            o = o.smooth(0.3)
        s.objects.append(o)
    cam = look_at((0.0, 3.2, -9.0), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), radians(50.0))
    return s, cam


def planes_scene(width=64, height=36):
    """A room of axis-aligned planes (normals +-x, +-y, -z; offsets positive, negative, +0 and -0;
    translated and scaled objects) with a tilted plane and spheres in it: the specialised field
    evaluates axis planes as one addition, which must give the interpreter's bits everywhere."""
    s = Scene(width, height)
    s.materials = [Material((0.8, 0.8, 0.8)), Material((0.7, 0.3, 0.2)), Material((0.2, 0.5, 0.7))]
    s.objects = [
        Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, 0),
        Object(Prim.plane((0.0, -1.0, 0.0), 4.0), Transform.IDENTITY, 1),
        Object(Prim.plane((1.0, 0.0, 0.0), 5.0), Transform((0.25, 0.0, 0.0)), 2),
        Object(Prim.plane((-1.0, 0.0, 0.0), -0.0), Transform((5.5, 0.0, 0.0)), 1),
        Object(Prim.plane((0.0, 0.0, -1.0), 6.0), Transform((0.0, 0.0, 0.5), scale=2.0), 2),
        Object(Prim.plane((0.0, 0.6, 0.8), 2.5), Transform.IDENTITY, 0),
        Object(Prim.sphere(0.8), Transform((-1.0, 0.8, 0.0)), 1),
        Object(Prim.sphere(0.6), Transform((1.2, 0.6, 1.0)), 2),
    ]
    cam = look_at((0.0, 2.0, -9.0), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), radians(60.0))
    return s, cam


def unbounded_mix_scene(seed, width=64, height=36):
    """Objects the reference leaves unbounded (bend, repeat) as smooth-union and subtracted
    segments and as union members, CSG objects among them, after bounded ones on a plane: the
    specialised field skips their exact fields where their weak bounds clear the threshold."""
    from mm3e_cuda.scene import Expr

    rng = np.random.default_rng(seed)
    s = Scene(width, height)
    s.materials = [Material((0.8, 0.8, 0.8)), Material((0.7, 0.3, 0.2)), Material((0.2, 0.5, 0.7))]
    s.objects = [Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, 0)]
    for k in range(14):
        pos = tuple(float(v) for v in rng.uniform([-4, 0.5, -3], [4, 2.0, 3]))
        rot = mat3_from_euler(*rng.uniform(-1.2, 1.2, 3))
        if k % 3 == 0:
            e = Expr.union(Expr.sphere(float(rng.uniform(0.2, 0.5))),
                           Expr.transform(Expr.box(tuple(float(v) for v in rng.uniform(0.15, 0.4, 3))),
                                          Transform(tuple(float(v) for v in rng.uniform(-0.3, 0.3, 3)), rot, 0.9)))
            prim = Prim.csg(s.csg(e))
        elif k % 3 == 1:
            prim = Prim.cone(float(rng.uniform(0.3, 0.6)), float(rng.uniform(0.05, 0.2)), float(rng.uniform(0.6, 1.2)))
        else:
            prim = Prim.box(tuple(float(v) for v in rng.uniform(0.2, 0.5, 3)))
        o = Object(prim, Transform(pos, rot, float(rng.uniform(0.8, 1.2))), 1 + k % 2)
        o = o.bend(float(rng.uniform(-0.4, 0.4))) if k % 2 == 0 else o.repeat((float(rng.uniform(3.0, 5.0)), 0.0, 0.0))
        if k % 4 == 1:
            o = o.smooth(float(rng.uniform(0.1, 0.4)))
        elif k % 4 == 3:
            o = o.subtract()
        s.objects.append(o)
    cam = look_at((0.0, 3.0, -9.0), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), radians(55.0))
    return s, cam
