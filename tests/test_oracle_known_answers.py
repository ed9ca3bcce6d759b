"""The CPU oracle against the reference's own known answers and shipped renders.

Each test restates a check from the reference's test suite (file:line in the MM3E repository)
against the oracle, so the oracle is pinned before it checks the CUDA path.
"""
import math
import os

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from mm3e_cuda import abi, scenes
from mm3e_cuda.scene import (Expr, GiVolume, Light, Material, Object, Prim, Scene, SdfVolume, Transform,
                             normalize_f32)

F32 = np.float32
HERE = os.path.dirname(os.path.abspath(__file__))
NIL = 0xFFFFFFFF


def close(a, b, eps):
    return abs(a - b) <= eps


def field_scene(obj, n_mat=8):
    s = Scene(8, 8)
    for _ in range(n_mat):
        s.material(Material())
    s.add(obj)
    return s


def march(scene, origin, direction, subitize=0.0, secant=False, normals=False):
    scene.marcher.subitize = subitize
    scene.marcher.secant = secant
    rays = np.array([list(origin) + list(direction)], np.float32)
    return oracle_py.march_rays(scene.desc(), rays, threads=1, normals=normals)


# ---- mm3e-kit/tests/march_sign_crossing.rs:7-47 -------------------------------------------

def test_accelerated_sign_crossing_returns_plane_surface():
    s = field_scene(Object(Prim.plane((0.0, 0.0, 1.0), 0.0), Transform.IDENTITY, 7))
    for subitize in (0.0, 0.6):
        for secant in (False, True):
            for x in (0.0, 0.1, 0.5):
                d = normalize_f32((x, 0.0, -1.0))
                t, m, _ = march(s, (0.0, 0.0, 3.0), d, subitize, secant)
                expected = 3.0 / -d[2]
                assert m[0] == 7
                assert abs(t[0] - expected) < 0.002
                z = F32(3.0) + F32(d[2]) * F32(t[0])
                assert -0.00001 <= z < 0.002


def test_touching_sphere_bounds_do_not_authorize_negative_hit():
    s = field_scene(Object(Prim.sphere(1.0), Transform.IDENTITY, 3))
    t, m, _ = march(s, (0.0, 0.0, 2.0), (0.0, 0.0, -1.0))
    assert m[0] == 3 and abs(t[0] - 1.0) < 0.00001


def test_origin_inside_solid_is_immediate_hit():
    s = field_scene(Object(Prim.plane((0.0, 0.0, 1.0), 0.0), Transform.IDENTITY, 4))
    t, m, steps = march(s, (0.0, 0.0, -0.5), (0.0, 0.0, -1.0))
    assert m[0] == 4 and t[0] == 0.0 and steps[0] == 0


# ---- mm3e-kit/tests/kit.rs -----------------------------------------------------------------

def test_sdf_values_and_signs():
    assert close(oracle_py.sdf(abi.PRIM_SPHERE, [1.0], (2, 0, 0)), 1.0, 1e-5)
    assert close(oracle_py.sdf(abi.PRIM_SPHERE, [1.0], (0, 0, 0)), -1.0, 1e-5)
    assert close(oracle_py.sdf(abi.PRIM_BOX, [1, 1, 1], (2, 0, 0)), 1.0, 1e-5)
    assert close(oracle_py.sdf(abi.PRIM_TORUS, [1.0, 0.3], (1, 0, 0)), -0.3, 1e-5)
    assert oracle_py.sdf(abi.PRIM_CONE, [0.5, 0.2, 1.0], (0, 0, 0)) < 0
    assert oracle_py.sdf(abi.PRIM_CONE, [0.5, 0.2, 1.0], (3, 0, 0)) > 0
    assert oracle_py.sdf(abi.PRIM_ELLIPSOID, [1.0, 2.0, 0.5], (0, 0, 0)) < 0
    assert oracle_py.sdf(abi.PRIM_OCTAHEDRON, [1.0], (0, 0, 0)) < 0
    assert oracle_py.sdf(abi.PRIM_OCTAHEDRON, [1.0], (3, 3, 3)) > 0
    assert oracle_py.sdf(abi.PRIM_HEX_PRISM, [1.0, 1.0], (0, 0, 0)) < 0
    assert oracle_py.sdf(abi.PRIM_HEX_PRISM, [1.0, 1.0], (3, 0, 0)) > 0


def _grad_mag(kind, params, p, h=1e-3):
    g = []
    for k in range(3):
        a = list(p)
        b = list(p)
        a[k] += h
        b[k] -= h
        g.append((oracle_py.sdf(kind, params, a) - oracle_py.sdf(kind, params, b)) / (2 * h))
    return math.sqrt(sum(x * x for x in g))


def test_sdf_lipschitz_outside():
    assert close(_grad_mag(abi.PRIM_SPHERE, [1.0], (2.0, 0.3, -0.4)), 1.0, 1e-2)
    assert close(_grad_mag(abi.PRIM_BOX, [1, 1, 1], (2.0, 0.5, 0.3)), 1.0, 2e-2)
    assert close(_grad_mag(abi.PRIM_TORUS, [1.0, 0.3], (2.0, 0.2, 0.0)), 1.0, 2e-2)


def test_csg_union_subtract_intersect():
    a, b = (0.5, 1), (-0.3, 2)
    d, m = oracle_py.combine(0, a, b)
    assert m == 2 and close(d, -0.3, 1e-6)
    d, _ = oracle_py.combine(1, a, b)
    assert close(d, 0.5, 1e-6)
    d, m = oracle_py.combine(2, a, b)
    assert close(d, 0.5, 1e-6) and m == 1


def test_smooth_union_bounded_below_hard_union():
    a, b = (0.4, 1), (0.5, 2)
    hard = oracle_py.combine(0, a, b)[0]
    soft = oracle_py.combine(3, a, b, 0.3)[0]
    assert soft <= hard + 1e-6 and soft >= hard - 0.3
    assert close(oracle_py.combine(3, a, b, 0.0)[0], hard, 1e-6)


def test_domain_ops():
    q = oracle_py.domain(3, (2.6, -3.1, 0.2), 1.0, 1.0, 1.0)
    assert abs(q[0]) <= 0.5 + 1e-5 and abs(q[1]) <= 0.5 + 1e-5
    assert close(oracle_py.domain(0, (0.7, 0, 0), 0.2)[0], 0.5, 1e-6)
    assert close(oracle_py.domain(1, (0.0, 0, 0), 0.1)[0], -0.1, 1e-6)
    assert oracle_py.domain(6, (-2.0, 1.0, -3.0), 1.0, 0.0, 1.0) == (2.0, 1.0, 3.0)


def test_marcher_hits_sphere_and_normal_points_back():
    s = field_scene(Object(Prim.sphere(1.0), Transform.at((0.0, 0.0, -5.0)), 0))
    t, m, _, n = march(s, (0.0, 0.0, 0.0), (0.0, 0.0, -1.0), normals=True)
    assert m[0] == 0 and close(t[0], 4.0, 1e-2) and n[0][2] > 0.9


def test_boosted_steps_never_accept_buried_hits():
    s = field_scene(Object(Prim.sphere(1.0), Transform.IDENTITY, 0).onion(0.02))
    for subitize in (0.0, 0.6):
        s.marcher.subitize = subitize
        rays = []
        for iy in range(-12, 13):
            for ix in range(-12, 13):
                d = normalize_f32((ix * 0.02, iy * 0.02, -1.0))
                rays.append([0.0, 0.0, 5.0] + list(d))
        rays = np.array(rays, np.float32)
        t, m, _ = oracle_py.march_rays(s.desc(), rays, threads=1)
        hit = m != NIL
        assert hit.sum() > 100
        pos = rays[hit, :3] + rays[hit, 3:] * t[hit, None].astype(np.float32)
        d, _ = oracle_py.field(s.desc(), pos.astype(np.float32))
        eps = 0.0006 * (1.0 + t[hit] * 0.5)
        assert np.all(d > -2.0 * eps)


def test_shading_invariants():
    b = oracle_py.brdf((0, 1, 0), (0, 1, 0), (0, 1, 0), (0.8, 0.8, 0.8), 0.0, 0.3, 0.5)
    assert min(b) >= 0.0
    assert oracle_py.fresnel(1.0, 0.04) < oracle_py.fresnel(0.0, 0.04)
    t = oracle_py.aces((20.0, 20.0, 20.0))
    assert 0.0 <= t[0] <= 1.0


def test_sdf_volume_sampling_and_bad_layout():
    """kit.rs:244-262: trilinear interior value and conservative outside bound."""
    vol = SdfVolume((2, 2, 2), (0, 0, 0), (1, 1, 1), [0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0])
    s = Scene(8, 8)
    vid = s.volume(vol)
    s.add(Object(Prim.volume(vid), Transform.IDENTITY, 0))
    d, _ = oracle_py.field(s.desc(), np.array([[0.5, 0.25, 0.75]], np.float32))
    assert close(float(d[0]), 0.5, 1e-6)
    assert vol.recommended_normal_h() > 0.5
    assert s.marcher.normal_h >= vol.recommended_normal_h()


def test_sdfv_roundtrip_and_rejects_bad_input():
    """kit.rs:264-296."""
    vol = SdfVolume((2, 2, 2), (-1.0, -2.0, -3.0), (0.5, 0.75, 1.25), [0.0, 0.5, 1.0, 1.5, -0.25, 0.25, 0.75, 1.25])
    b = vol.to_sdfv_bytes()
    assert b[:8] == b"MM3ESDF1"
    r = SdfVolume.from_sdfv_bytes(b)
    assert r.dims == vol.dims and r.min == vol.min and r.cell == vol.cell and np.array_equal(r.data, vol.data)
    with pytest.raises(ValueError):
        SdfVolume.from_sdfv_bytes(b[:12])
    with pytest.raises(ValueError):
        SdfVolume.from_sdfv_bytes(b"X" + b[1:])


# ---- mm3e-orchestrator/tests/engine.rs ------------------------------------------------------

def _gi_scene(vmin, vmax, dims, radiance):
    """GiVolume::bake with a closure-free radiance: cubes built as the bake builds them for
    samples = 1 (one axis direction of weight 1, so each face is the radiance itself)."""
    nx, ny, nz = (max(1, d) for d in dims)
    size = [F32(b) - F32(a) for a, b in zip(vmin, vmax)]
    cell = [F32(size[i]) / F32(max(n, 2) - 1) for i, n in enumerate((nx, ny, nz))]
    cubes = np.zeros((nz, ny, nx, 6, 3), np.float32)
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                probe = (F32(vmin[0]) + F32(i) * cell[0], F32(vmin[1]) + F32(j) * cell[1],
                         F32(vmin[2]) + F32(k) * cell[2])
                cubes[k, j, i, :, :] = radiance(probe)
    s = Scene(8, 8)
    s.gi = GiVolume(vmin, size, (nx, ny, nz), cubes)
    return s


def test_gi_volume_interpolates_known_field():
    """engine.rs:145-156: a radiance linear in x is reproduced by trilinear interpolation."""
    s = _gi_scene((0.0, 0.0, 0.0), (4.0, 2.0, 4.0), (5, 3, 5), lambda o: [o[0]] * 3)
    out = oracle_py.gi_sample(s.desc(), [[2.0, 1.0, 2.0], [2.5, 1.0, 2.0]], [[1, 0, 0], [1, 0, 0]])
    assert abs(out[0][0] - 2.0) < 1e-3 and abs(out[1][0] - 2.5) < 1e-3


def test_gi_degenerate_dims_do_not_panic():
    """engine.rs:158-166."""
    for dims in ((0, 5, 6), (1, 1, 1), (3, 0, 3)):
        s = _gi_scene((0.0, 0.0, 0.0), (4.0, 4.0, 4.0), dims, lambda o: [0.5] * 3)
        out = oracle_py.gi_sample(s.desc(), [[2.0, 2.0, 2.0]], [[0.0, 1.0, 0.0]])
        assert np.all(np.isfinite(out))


def test_accelerated_field_matches_linear_fold():
    """engine.rs:422-449 (volume + smooth sphere) and the reference's gallery: the BVH world
    equals the linear reference fold."""
    s, _ = scenes.canonical_asset_scene()
    s.add(Object(Prim.sphere(0.35), Transform.at((0.7, 0.35, 0.0)), 1).smooth(0.18))
    g, _ = scenes.reference_gallery_scene()
    rng = np.random.default_rng(3)
    for scene in (s, g):
        pts = rng.uniform(-4, 4, size=(4000, 3)).astype(np.float32)
        a, am = oracle_py.field(scene.desc(), pts)
        b, bm = oracle_py.field(scene.desc(), pts, linear=True)
        assert np.all(np.abs(a - b) < 1e-5 + 1e-6 * np.abs(b))
        near = np.abs(b) < 2.0
        assert np.array_equal(am[near], bm[near])


def test_render_is_deterministic_across_worker_counts():
    """engine.rs:84-91 and canonical.rs:192-203: identical pixels for 1 and 4 workers."""
    s, cam = scenes.demo_scene()
    a = oracle_py.render(s.desc(), cam, threads=1)
    b = oracle_py.render(s.desc(), cam, threads=4)
    assert np.array_equal(a, b)
    fb = mm3e_cuda.to_rgba8(a)
    assert np.any(fb[..., :3] != fb[0, 0, :3])  # not a flat image (engine.rs:93-104)


def test_all_render_modes_run():
    """engine.rs:117-133."""
    s, cam = scenes.demo_scene()
    for mode in range(6):
        s.mode = mode
        fb = oracle_py.render(s.desc(), cam, threads=2)
        assert fb.shape == (64, 96, 4) and np.all(np.isfinite(fb))


# ---- committed oracle fixtures and the reference's shipped renders ---------------------------

def test_oracle_reproduces_committed_frames():
    from golden.make_fixtures import parity_scenes
    frames = np.load(os.path.join(HERE, "golden", "oracle_frames.npz"))
    for name, fn in parity_scenes().items():
        s, cam = fn()
        got = mm3e_cuda.to_rgba8(oracle_py.render(s.desc(), cam, threads=2))[..., :3]
        assert np.array_equal(got, frames[name]), name


REFERENCE_DIR = os.environ.get("MM3E_REFERENCE_DIR", "")


@pytest.mark.skipif(not (REFERENCE_DIR and os.path.exists(os.path.join(REFERENCE_DIR, "gallery.png"))),
                    reason="MM3E_REFERENCE_DIR (a checkout of the reference with its shipped renders) is not set")
def test_oracle_matches_reference_gallery_render():
    """The reference ships gallery.png, its own render of examples/gallery.rs."""
    from golden.tests_png import read_png
    s, cam = scenes.reference_gallery_scene()
    ours = mm3e_cuda.to_rgba8(oracle_py.render(s.desc(), cam))[..., :3].astype(np.int32)
    ref = read_png(os.path.join(REFERENCE_DIR, "gallery.png"))[..., :3].astype(np.int32)
    d = np.abs(ours - ref).max(-1)
    assert (d == 0).mean() >= 0.985
    assert (d <= 1).mean() >= 0.999
