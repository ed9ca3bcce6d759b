"""C-ABI library checks that need no GPU: exports, host helpers, validation."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from mm3e_cuda import abi, scenes
from mm3e_cuda.native import LIB_PATH, lib
from mm3e_cuda.scene import Expr, Material, Object, Prim, Scene, Transform

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "mm3e_cuda.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mm3e_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib()
    out = subprocess.check_output(["nm", "-D", "--defined-only", LIB_PATH]).decode()
    exported = set(re.findall(r" T (mm3e_\w+)", out))
    declared = header_functions()
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    assert sorted(abi.EXPORTED_SYMBOLS) == declared


def test_abi_version():
    assert lib().mm3e_abi_version() == abi.ABI_VERSION


def test_struct_sizes_match_header():
    # sizes the C compiler gives the header's structs (x86_64 / aarch64 LP64 agree)
    assert C.sizeof(abi.Object) == 4 * 4 + 4 + 7 * 4 + 9 * 4 + 3 * 4 + 4 + 4 + 3 * 4 + 4 + 4 + 3 * 4 + 4 + 4
    assert C.sizeof(abi.Material) == 11 * 4
    assert C.sizeof(abi.Camera) == 13 * 4
    assert C.sizeof(abi.DynSphere) == 8 * 4


@pytest.mark.parametrize("eye,target,fov", [((0, 2, -7), (0, 1, 0), 45.0), ((3.5, 1.2, -2.0), (0.1, 0.7, 0.3), 52.0),
                                            ((0, 0, 5), (0, 0, 0), 30.0)])
def test_look_at_matches_oracle_bitwise(eye, target, fov):
    fov_r = mm3e_cuda.radians(fov)
    a = mm3e_cuda.look_at(eye, target, (0.0, 1.0, 0.0), fov_r)
    b = abi.Camera()
    F3 = C.c_float * 3
    oracle_py.lib().oracle_camera_look_at(F3(*eye), F3(*target), F3(0.0, 1.0, 0.0), fov_r, C.byref(b))
    assert bytes(a) == bytes(b)


@pytest.mark.parametrize("yaw,pitch,radius", [(0.55, 0.32, 8.5), (-7.0, 1.7, 3.0), (100.0, -0.2, -4.0)])
def test_orbit_camera_matches_oracle_bitwise(yaw, pitch, radius):
    tgt = (0.2, 0.85, 0.4)
    a = mm3e_cuda.orbit_camera(tgt, radius, yaw, pitch, mm3e_cuda.radians(50.0))
    b = abi.Camera()
    oracle_py.lib().oracle_orbit_camera((C.c_float * 3)(*tgt), radius, yaw, pitch, mm3e_cuda.radians(50.0), C.byref(b))
    assert bytes(a) == bytes(b)


def test_euler_rotation_matches_oracle_bitwise():
    for ang in ((0.0, 0.6, 0.0), (1.2, 0.0, 0.2), (0.3, -0.7, 2.1)):
        a = mm3e_cuda.mat3_from_euler(*ang)
        out = (C.c_float * 9)()
        oracle_py.lib().oracle_mat3_from_euler(*ang, out)
        assert np.array_equal(np.array(a, np.float32), np.array(list(out), np.float32))


def test_quat_rotation_matches_oracle_bitwise():
    """Quat::to_mat3 (vec.rs:318-326, after Quat::normalize at :276-283), which places the seeded
    procedural scenes' objects: the library's helper against the oracle's restatement, bit for
    bit, on random quaternions and on zero, tiny and unnormalised ones."""
    rng = np.random.default_rng(5)
    qs = [q for q in rng.normal(size=(300, 4)).astype(np.float32)]
    qs += [np.array(v, np.float32) for v in ((0, 0, 0, 0), (1e-13, 0, 0, 0), (0, 0, 0, -2), (3e-7, 1e-7, 2e-7, 4e-7),
                                              (1e20, -3e19, 2e19, 5e19), (0.5, 0.5, 0.5, 0.5))]
    for q in qs:
        a = np.array(mm3e_cuda.quat_to_mat3(tuple(float(v) for v in q)), np.float32)
        out = (C.c_float * 9)()
        oracle_py.lib().oracle_quat_to_mat3((C.c_float * 4)(*q), out)
        b = np.array(list(out), np.float32)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (q, a, b)


def _scene_bits(scene, cam):
    rows = [bytes(cam)]
    for o in scene.objects:
        rows.append(np.array(o.xform.rot + o.xform.pos + (o.xform.scale,), np.float32).tobytes())
    return rows


def test_oracle_host_math_builds_identical_scenes():
    """Scenes and cameras built through the oracle's helpers (the CPU reference arm's route, which
    must not load the CUDA library) hold the same binary32 values as those built through the
    library's helpers."""
    from mm3e_cuda.scene import use_host_math

    builders = [lambda: scenes.gallery_scene(64, 36), lambda: scenes.spheres_scene(64, 36),
                lambda: scenes.cornell_scene(64, 36), lambda: scenes.procedural_scene(3, 64, 36),
                lambda: scenes.procedural_scene(17, 64, 36)]
    for build in builders:
        a = _scene_bits(*build())
        prev = use_host_math(oracle_py.HostMath())
        try:
            b = _scene_bits(*build())
        finally:
            use_host_math(prev)
        assert a == b


def test_reference_arm_loads_no_cuda_library():
    """bench.py --impl reference builds its scene and camera and times the oracle without mapping
    libmm3e_cuda.so into the process (checked in a child process's memory map)."""
    code = ("import sys, os; sys.path.insert(0, os.path.join(%r, 'atom-3d-engine_gb300')); "
            "sys.path.insert(0, os.path.join(%r, 'oracle')); import oracle_py; "
            "from mm3e_cuda.scene import use_host_math; use_host_math(oracle_py.HostMath()); "
            "from mm3e_cuda import scenes; s, c = scenes.gallery_scene(32, 18); scenes.procedural_scene(4, 32, 18); "
            "oracle_py.render(s.desc(), c, threads=2); "
            "maps = open('/proc/self/maps').read(); "
            "print('cuda' if 'libmm3e_cuda' in maps else 'clean', 'oracle' if 'liboracle_mm3e' in maps else '')"
            ) % (ROOT, ROOT)
    out = subprocess.check_output([os.sys.executable, "-c", code]).decode().split()
    assert out == ["clean", "oracle"], out


def test_row_bands_follow_reference_split():
    from mm3e_cuda.replicas import bands
    assert bands(4, 10) == [(0, 3), (3, 6), (6, 8), (8, 10)]
    assert bands(3, 2) == [(0, 1), (1, 2)]
    for world in (1, 2, 3, 7):
        b = bands(world, 1080)
        assert b[0][0] == 0 and b[-1][1] == 1080
        assert all(b[i][1] == b[i + 1][0] for i in range(len(b) - 1))


def _validate(scene):
    return mm3e_cuda.validate(scene)


def test_valid_scenes_validate():
    for fn in (scenes.spheres_scene, scenes.gallery_scene, scenes.hero_scene, scenes.demo_scene,
               scenes.canonical_asset_scene, lambda: scenes.procedural_scene(5)):
        s, _ = fn()
        assert _validate(s) == (abi.OK, "")


def test_invalid_scenes_are_rejected():
    s = Scene(16, 16)
    s.materials = []
    assert _validate(s)[0] == abi.ERR_INVALID  # appearance.rs:251-253
    s, _ = scenes.canonical_scene()
    s.add(Object(Prim.surface(0), Transform.IDENTITY, 0))
    code, msg = _validate(s)
    assert code == abi.ERR_UNSUPPORTED and "surface" in msg  # wgsl.rs:45-47
    s, _ = scenes.canonical_scene()
    s.width = 20000
    assert _validate(s)[0] == abi.ERR_INVALID  # mm3e-gpu/src/lib.rs:139-141
    s, _ = scenes.canonical_scene()
    s.add(Object(Prim.sphere(float("nan")), Transform.IDENTITY, 0))
    assert _validate(s)[0] == abi.ERR_INVALID


def test_bloom_radius_limit():
    """A blooming scene's blur radius is capped at 4096 (each pass sums 2r+1 taps per pixel); the
    radius of a scene without bloom is not looked at."""
    s, _ = scenes.gallery_scene(32, 18)
    s.post.bloom_radius = 4096
    assert _validate(s) == (abi.OK, "")
    s.post.bloom_radius = 4097
    code, msg = _validate(s)
    assert code == abi.ERR_UNSUPPORTED and "bloom radius" in msg
    s.post.bloom = False
    assert _validate(s) == (abi.OK, "")
    s.post.bloom = True
    s.post.bloom_intensity = 0.0
    assert _validate(s) == (abi.OK, "")


@pytest.mark.parametrize("expr", [
    Expr.sphere(float("nan")),
    Expr.plane((0.0, 2.0, 0.0), 0.0),
    Expr.capsule((0, 0, 0), (0, 0, 0), 1.0),
    Expr.transform(Expr.sphere(1.0), Transform((0, 0, 0), (1, 0, 0, 0, 1, 0, 0, 0, 1), 0.0)),
])
def test_malformed_csg_rejected(expr):
    """csg.rs:174-195 (malformed_geometry_and_excessive_expression_depth_are_rejected)."""
    s, _ = scenes.canonical_scene()
    eid = s.csg(expr)
    s.add(Object(Prim.csg(eid), Transform.IDENTITY, 0))
    assert _validate(s)[0] == abi.ERR_INVALID


def test_csg_depth_budget_and_cumulative_scale():
    s, _ = scenes.canonical_scene()
    deep = Expr.sphere(1.0)
    for _ in range(64):
        deep = Expr.offset(deep, 0.01)
    s.add(Object(Prim.csg(s.csg(deep)), Transform.IDENTITY, 0))
    assert _validate(s)[0] == abi.ERR_INVALID
    s, _ = scenes.canonical_scene()
    huge = Expr.ellipsoid((1.0, 1.0, 1.0))
    for _ in range(8):
        huge = Expr.transform(huge, Transform((0, 0, 0), (1, 0, 0, 0, 1, 0, 0, 0, 1), 1000.0))
    s.add(Object(Prim.csg(s.csg(huge)), Transform.IDENTITY, 0))
    assert _validate(s)[0] == abi.ERR_INVALID


def test_valid_csg_accepted_and_tape_sized():
    s, _ = scenes.canonical_asset_scene()
    assert _validate(s)[0] == abi.OK
    n = C.c_size_t()
    assert lib().mm3e_scene_tape_bytes(s.desc().ptr, C.byref(n)) == abi.OK
    assert n.value > 0 and n.value % 16 == 0


def test_scene_tape_bytes_on_the_host():
    """mm3e_scene_tape: the lowered tape without a device. Its size equals mm3e_scene_tape_bytes,
    it starts with the tape header (magic, byte count), lowering is deterministic, a short buffer
    takes a prefix, a NULL buffer only reports the size, and an invalid scene is rejected."""
    s, _ = scenes.canonical_asset_scene()
    h = s.desc()
    n = C.c_size_t()
    assert lib().mm3e_scene_tape_bytes(h.ptr, C.byref(n)) == abi.OK
    size = C.c_size_t()
    assert lib().mm3e_scene_tape(h.ptr, None, 0, C.byref(size)) == abi.OK
    assert size.value == n.value
    buf = (C.c_uint8 * n.value)()
    assert lib().mm3e_scene_tape(h.ptr, buf, n.value, C.byref(size)) == abi.OK
    tape = bytes(buf)
    magic, nbytes = np.frombuffer(tape[:8], np.uint32)
    assert magic == 0x4D334554 and nbytes == n.value
    assert mm3e_cuda.scene_tape(s) == tape
    short = (C.c_uint8 * 64)()
    assert lib().mm3e_scene_tape(h.ptr, short, 64, C.byref(size)) == abi.OK
    assert bytes(short) == tape[:64] and size.value == n.value
    bad, _ = scenes.canonical_scene()
    bad.materials = []
    assert lib().mm3e_scene_tape(bad.desc().ptr, None, 0, C.byref(size)) == abi.ERR_INVALID


def test_context_without_gpu_fails_cleanly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(mm3e_cuda.RenderError) as e:
        mm3e_cuda.Context(0)
    assert e.value.code == abi.ERR_CUDA
