"""Weak-bound culls of the specialised field never skip a member that could win.

For a union member that the exact bounding-sphere test never culls (the reference's unbounded
objects: bend, repeat; and the fields that can undercut their spheres: ellipsoid, octahedron,
hexagonal prism), the generated field skips the exact evaluation where
    c * (n - R) * scale - post - (n + R) * scale * 2^-10 > best   (best >= 0)
with n the local point's norm over the non-repeating axes (weak_beyond in device_math.cuh). This
is only exact if the object's field is at least that bound everywhere. These tests take the
constants the generator emitted for each primitive under each modifier, replay the bound in
binary32 and check it against the oracle's field of the object (world field of a one-object
scene) on points all around it.
"""
import re

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from mm3e_cuda.scene import IDENTITY_ROT, Expr, Material, Object, Prim, Scene, Transform, mat3_from_euler

F = np.float32

PRIMS = {
    "sphere": Prim.sphere(0.7),
    "box": Prim.box((0.5, 0.9, 0.3)),
    "round_box": Prim.round_box((0.6, 0.4, 0.5), 0.15),
    "torus": Prim.torus(0.7, 0.2),
    "cylinder": Prim.cylinder(0.8, 0.4),
    "capsule": Prim.capsule((0.3, -0.5, 0.1), (0.4, 0.6, 0.0), 0.25),
    "cone": Prim.cone(0.6, 0.2, 1.2),
    "ellipsoid": Prim.ellipsoid((0.5, 0.9, 0.3)),
    "octahedron": Prim.octahedron(0.8),
    "hex_prism": Prim.hex_prism(0.6, 0.5),
}
MODS = {
    "bend": lambda o: o.bend(0.6),
    "repeat_x": lambda o: o.repeat((3.0, 0.0, 0.0)),
    "repeat_xz_twist": lambda o: o.repeat((2.5, 0.0, 3.0)).twist(0.8),
    "mirror_elongate_round": lambda o: o.mirror(True, False, True).elongate((0.3, 0.0, 0.2)).round(0.1),
    "onion_bend": lambda o: o.onion(0.05).bend(-0.4),
    "plain": lambda o: o,
}

_HEX = r"__uint_as_float\(0x([0-9a-f]+)u\)"
# the threshold of a weak test: bd in a union run; the accumulator's in a skippable one-object segment
_THR = r"(?:bd|-acc\.d|acc\.d|__fadd_ru\(acc\.d, __uint_as_float\(0x[0-9a-f]+u\)\))"


def _f(h):
    return np.array([int(h, 16)], np.uint32).view(F)[0]


def _scene(obj, with_anchor):
    s = Scene(32, 32)
    s.materials = [Material((0.8, 0.8, 0.8))]
    s.objects = [obj]
    if with_anchor:  # a far sphere so that the object sits in a LINEAR union run
        s.objects.append(Object(Prim.sphere(0.1), Transform((40.0, 40.0, 40.0)), 0))
    return s


def _weak_constants(src):
    """(rot, pos, inv, axes, R, c, scale, post, sq) of the one weak-bound cull in `src`; sq holds the
    (A, B) constants of the square-root-free form, or None for the plain form."""
    m = re.search(r"const float RO\[9\] = \{([^}]*)\};", src)
    if m:
        rot = np.array([_f(h) for h in re.findall(r"0x([0-9a-f]+)u", m.group(1))], F)
        local = r"rot_t_fma\(RO, p - V\{" + _HEX + ", " + _HEX + ", " + _HEX + r"\}\)"
    else:  # an identity rotation is left out of the test
        rot = None
        local = r"p - V\{" + _HEX + ", " + _HEX + ", " + _HEX + r"\}"
    head = r"\(scale\(" + local + ", " + _HEX + r"\), (true|false), (true|false), (true|false), "
    sq = re.search(r"weak_beyond_sq" + head + _HEX + ", " + _HEX + ", " + _THR + r"\) /\* weak bound R c scale post: " +
                   " ".join([_HEX] * 4), src)
    if sq:
        g = sq.groups()
        consts = (_f(g[9]), _f(g[10]), _f(g[11]), _f(g[12]))
        ab = (_f(g[7]), _f(g[8]))
    else:
        call = re.search(r"weak_beyond" + head + ", ".join([_HEX] * 4) + ", " + _THR + r"\)", src)
        assert call, "no weak-bound cull emitted"
        g = call.groups()
        consts = tuple(_f(x) for x in g[7:11])
        ab = None
    pos = np.array([_f(g[0]), _f(g[1]), _f(g[2])], F)
    inv = _f(g[3])
    axes = [g[4] == "true", g[5] == "true", g[6] == "true"]
    return (rot, pos, inv, axes) + consts + (ab,)


def _fma32(a, b, c):
    """fl(a b + c): the product is exact in binary64; the sum rounds there and then to binary32
    (a double rounding that can differ from one fused rounding by a unit in rare ties, far
    inside the margins tested here)."""
    return F(np.float64(a) * np.float64(b) + np.float64(c))


def _local_n2(pts, rot, pos, inv, axes, fused=False):
    """The squared norm of the local point over the kept axes, as the generated test computes it:
    the rotation with fused multiply-adds (rot_t_fma; none for the identity), then the sum of
    squares in weak_beyond's order, or with fused multiply-adds for weak_beyond_sq (fused)."""
    d = (pts - pos).astype(F)
    if rot is None:
        l = d
    else:
        l = np.stack([_fma32(rot[3 * k], d[:, 0], _fma32(rot[3 * k + 1], d[:, 1], F(rot[3 * k + 2] * d[:, 2])))
                      for k in range(3)], axis=1)
    l = (l * inv).astype(F)
    if fused:
        n2 = F(l[:, 2] * l[:, 2]) if axes[2] else np.zeros(len(pts), F)
        for a in (1, 0):
            if axes[a]:
                n2 = _fma32(l[:, a], l[:, a], n2)
        return n2
    n2 = np.zeros(len(pts), F)
    for a in range(3):
        n2 = F(n2 + (F(l[:, a] * l[:, a]) if axes[a] else F(0)))
    return n2


def _bound(pts, rot, pos, inv, axes, R, c, scl, post):
    """weak_beyond's bound minus its margin, in binary32 with the device's operation order."""
    n = np.sqrt(_local_n2(pts, rot, pos, inv, axes)).astype(F)
    lb = F(F(F(F(n - R) * c) * scl) - post)
    return F(lb - F(F(F(n + R) * scl) * F(0.0009765625)))


@pytest.mark.parametrize("rotated", [True, False])
@pytest.mark.parametrize("mod", list(MODS))
@pytest.mark.parametrize("prim", list(PRIMS))
def test_weak_bound_holds(prim, mod, rotated):
    rng = np.random.default_rng(abs(hash((prim, mod, rotated))) % (1 << 32))
    rot = mat3_from_euler(0.3, -0.7, 1.1) if rotated else IDENTITY_ROT
    base = Object(PRIMS[prim], Transform((0.4, 1.2, -0.6), rot, 1.3), 0)
    obj = MODS[mod](base)
    src = mm3e_cuda.spec_source(_scene(obj, True))
    weak = "weak_beyond" in src
    bounded_conservative = prim not in ("ellipsoid", "octahedron", "hex_prism") and mod not in (
        "bend", "repeat_x", "repeat_xz_twist", "onion_bend")
    if bounded_conservative:
        assert not weak  # the exact sphere test covers it
        return
    assert weak
    _check_bound(src, lambda: _scene(obj, False), rng)


def _check_bound(src, field_scene, rng, centre=(0.4, 1.2, -0.6)):
    """The weak test's constants in `src` against the oracle's field of `field_scene()` (the object
    alone) on points all around `centre`: the bound never exceeds the field, it is not vacuous,
    and the square-root-free form culls only where the plain bound clears the threshold."""
    *consts, ab = _weak_constants(src)
    d = rng.standard_normal((40000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.uniform(0.0, 6.0, 40000) ** 1.5
    pts = (np.array(centre) + d * r[:, None]).astype(F)
    field, _ = oracle_py.field(field_scene().desc(), pts)
    lb = _bound(pts, *consts)
    live = lb >= 0
    assert live.mean() > 0.2  # the bound is not vacuous
    bad = live & ~(field >= lb)
    assert not bad.any(), (pts[bad][:3], field[bad][:3], lb[bad][:3])
    if ab is None:
        return
    # the square-root-free form: constants no smaller than the exact ones, and on thresholds bd
    # around the bound every cull it makes is one the plain form makes, with the field above bd
    rot, pos, inv, axes, R, c, scl, post = consts
    A, B = ab
    K = float(scl) * (float(c) - 2.0 ** -10)
    assert K > 0 and A >= float(post) + float(R) * float(scl) * (float(c) + 2.0 ** -10)
    assert B >= (1.0 + 2.0 ** -17) / K
    n2 = _local_n2(pts, rot, pos, inv, axes, fused=True)
    for scale_bd in (0.5, 0.9, 0.99, 0.999, 1.0, 1.001):
        bd = np.maximum(lb * F(scale_bd), F(0)).astype(F)
        t = F(F(bd + A) * B)
        sq = n2 > F(t * t)
        assert not (sq & ~(lb > bd)).any()
        assert not (sq & ~(field > bd)).any()
    bd = (lb * F(0.98)).astype(F)
    assert (n2 > F(F(F(bd + A) * B) ** 2))[lb > 0.1].mean() > 0.5  # and it still culls


CSG_EXPRS = {
    "union_transform": lambda: Expr.union(Expr.sphere(0.5), Expr.transform(
        Expr.box((0.3, 0.6, 0.2)), Transform((0.4, 0.1, 0.0), mat3_from_euler(0.3, 0.2, 0.1), 0.8))),
    "smooth_shell": lambda: Expr.shell(Expr.smooth_union(Expr.torus(0.5, 0.15),
                                                         Expr.capsule((0, -0.4, 0), (0, 0.4, 0), 0.2), 0.3), 0.05),
    "intersect_offset": lambda: Expr.offset(Expr.intersect(Expr.box((0.6, 0.6, 0.6)), Expr.sphere(0.75)), 0.05),
    "subtract_scaled": lambda: Expr.subtract(Expr.transform(Expr.cylinder(0.5, 0.4), Transform((0.0, 0.0, 0.2),
                                                                                             IDENTITY_ROT, 1.3)),
                                             Expr.sphere(0.3)),
    "ellipsoid_octahedron": lambda: Expr.union(Expr.ellipsoid((0.5, 0.3, 0.4)), Expr.octahedron(0.5)),
    "negative_offset_cone": lambda: Expr.offset(Expr.cone(0.6, 0.2, 1.2), -0.1),
}


def _csg_scene(expr, mod, lead=None, combine=None):
    s = Scene(32, 32)
    s.materials = [Material((0.8, 0.8, 0.8))]
    obj = MODS[mod](Object(Prim.csg(s.csg(expr)), Transform((0.4, 1.2, -0.6), mat3_from_euler(0.2, -0.5, 0.9), 1.1), 0))
    if combine == "smooth":
        obj = obj.smooth(0.3)
    elif combine == "subtract":
        obj = obj.subtract()
    s.objects = ([lead] if lead is not None else []) + [obj]
    return s


@pytest.mark.parametrize("mod", ["bend", "repeat_x", "onion_bend"])
@pytest.mark.parametrize("expr", list(CSG_EXPRS))
def test_csg_weak_bound_holds(expr, mod):
    """A CSG object that the reference leaves unbounded (bend, repeat) gets a weak bound from its
    program's parts (csg_weak in spec_gen.cpp); the bound holds against the oracle's field."""
    rng = np.random.default_rng(abs(hash((expr, mod))) % (1 << 32))
    anchor = Object(Prim.sphere(0.1), Transform((40.0, 40.0, 40.0)), 0)
    s = _csg_scene(CSG_EXPRS[expr](), mod)
    s.objects.append(anchor)
    src = mm3e_cuda.spec_source(s)
    assert "weak_beyond" in src
    _check_bound(src, lambda: _csg_scene(CSG_EXPRS[expr](), mod), rng)


@pytest.mark.parametrize("combine", ["smooth", "subtract"])
@pytest.mark.parametrize("shape", ["bent_cone", "csg"])
def test_unbounded_one_object_segment_weak_skip(shape, combine):
    """An unbounded smooth-union or subtracted object (its own segment, after the accumulator of
    the objects before it) skips its exact field where its weak bound clears the accumulator's
    threshold; the bound holds against the oracle's field."""
    rng = np.random.default_rng(7 if shape == "csg" else 8)
    lead = Object(Prim.sphere(0.5), Transform((6.0, 0.5, 0.0)), 0)
    if shape == "csg":
        make = lambda with_lead: _csg_scene(CSG_EXPRS["union_transform"](), "bend", lead if with_lead else None,
                                            combine if with_lead else None)
    else:
        def make(with_lead):
            s = Scene(32, 32)
            s.materials = [Material((0.8, 0.8, 0.8))]
            o = Object(Prim.cone(0.6, 0.2, 1.2), Transform((0.4, 1.2, -0.6), mat3_from_euler(0.2, -0.5, 0.9), 1.1),
                       0).bend(-0.36)
            if with_lead:
                o = o.smooth(0.3) if combine == "smooth" else o.subtract()
            s.objects = ([lead] if with_lead else []) + [o]
            return s
    src = mm3e_cuda.spec_source(make(True))
    assert "// weak skip" in src
    _check_bound(src, lambda: make(False), rng)
