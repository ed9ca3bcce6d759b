"""The device field and the per-ray state machines, compiled for the host (host_checks.py).

Scene-specialised fields against the tape interpreter:

The specialised program (spec_gen.cpp's generated field: inlined objects, generated CSG programs,
axis planes, linearised and enclosing-sphere pre-tests, weak bounds and skips) and the
interpreter's world_eval (WorldPlan::eval, accel.rs:209-252) compile as plain C++ with the host
definitions of the device intrinsics in tests/host_field/host_shim.h. Both are evaluated on the
same binary32 points over the scene's lowered tape (mm3e_scene_tape), and their (distance,
material) pairs must agree bit for bit. This covers many seeded scenes without a GPU; the GPU
tests check the same identity on the device (test_gpu_spec.py)."""
import shutil
import subprocess
import zlib

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from host_checks import (CSRC, CUDA_INCLUDE, HOST_DIR, SCENES, SHIM, STUBS, compile_harnesses, harness_source,
                         spec_namespace)

MAIN = harness_source("field_check.inc")


def _points(scene, cam, rng, n=6000):
    """Points along the camera's rays at random distances, and points in a box around the scene:
    near surfaces, inside objects and far away."""
    eye = np.array(cam.eye, np.float64)
    fwd, right, up = (np.array(v, np.float64) for v in (cam.forward, cam.right, cam.up))
    sx, sy = rng.uniform(-1, 1, n // 2), rng.uniform(-1, 1, n // 2)
    d = fwd + np.outer(sx * cam.fov_scale * 1.7, right) + np.outer(sy * cam.fov_scale, up)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t = rng.uniform(0, 25, n // 2) ** 1.0
    on_rays = eye + d * t[:, None]
    box = rng.uniform([-8, -2, -8], [8, 6, 8], (n - n // 2, 3))
    # signed zeros, exact grid points, far points (up to 1e6: the identity is claimed for samples
    # whose squared coordinates stay finite in binary32, which a march of any sane extent keeps)
    special = np.array([[0.0, 0.0, 0.0], [-0.0, 0.0, -0.0], [1.0, 0.0, -1.0], [0.5, 0.25, 0.0], [3e3, -2e3, 1e3],
                        [1e6, 1.0, -1e6], [-4.0, 0.0, 4.0], [0.0, -6.0, 0.0]], np.float64)
    return np.concatenate([on_rays, box, special]).astype(np.float32)


@pytest.fixture(scope="module")
def field_exes(tmp_path_factory):
    """The field check of every scene, compiled in parallel."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    root = tmp_path_factory.mktemp("field")
    jobs = {}
    for name, make in SCENES.items():
        src = mm3e_cuda.spec_source(make()[0])
        body = src[src.index("namespace spec {") + len("namespace spec {"):src.index("struct Field_")]
        defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
        d = root / name
        d.mkdir()
        (d / "field.inc").write_text(body)
        (d / "main.cpp").write_text(defines + '#include "device_math.cuh"\n' + MAIN)
        jobs[name] = (d, ["-I", str(d), "-include", SHIM])
    return compile_harnesses(jobs, "field_check")


@pytest.mark.parametrize("name", list(SCENES))
def test_specialised_field_equals_interpreter_on_host(name, field_exes, tmp_path):
    scene, cam = SCENES[name]()
    exe = field_exes[name]
    (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    _points(scene, cam, np.random.default_rng(zlib.crc32(name.encode()))).tofile(tmp_path / "points.bin")
    r = subprocess.run([str(exe), str(tmp_path / "tape.bin"), str(tmp_path / "points.bin")], capture_output=True,
                       text=True)
    print(name, r.stdout.strip().splitlines()[-1] if r.stdout.strip() else r.stderr[-500:])
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]


INTERP_MAIN = harness_source("interp_field.inc")


@pytest.fixture(scope="module")
def interpreter_exe(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("interp")
    (d / "main.cpp").write_text('#include "device_math.cuh"\n' + INTERP_MAIN)
    exe = d / "interp"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, str(d / "main.cpp"), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("name", list(SCENES))
def test_interpreter_field_equals_oracle_on_host(name, interpreter_exe, tmp_path):
    """The device tape interpreter's world field (device_math.cuh world_eval), compiled for the
    host, against the oracle's restatement of Scene::field (oracle_field): bit for bit, distance
    and material, on the same points. On the host both call the same libm, so this pins the
    device field code's operation order to the oracle's; on the GPU only CUDA's own sinf/cosf and
    the like can differ, within the tolerance the GPU parity tests hold."""
    scene, cam = SCENES[name]()
    (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    pts = _points(scene, cam, np.random.default_rng(zlib.crc32(name.encode())))
    pts.tofile(tmp_path / "points.bin")
    subprocess.run([str(interpreter_exe), str(tmp_path / "tape.bin"), str(tmp_path / "points.bin"),
                    str(tmp_path / "out.bin")], check=True)
    out = np.fromfile(tmp_path / "out.bin", np.uint32).reshape(-1, 2)
    d, m = out[:, 0].view(np.float32), out[:, 1]
    od, om = oracle_py.field(scene.desc(), pts)
    same = (d.view(np.uint32) == od.view(np.uint32)) | (np.isnan(d) & np.isnan(od))
    assert same.all(), (pts[~same][:3], d[~same][:3], od[~same][:3])
    assert np.array_equal(m, om)


SHADE_MAIN = harness_source("shade_formulas.inc")


def test_shading_formulas_equal_oracle_on_host(tmp_path):
    """The device shading formulas (device_math.cuh brdf, fresnel_schlick and aces1; shade.rs:51-72
    and post.rs ACES), compiled for the host, against the oracle's restatements (oracle_brdf,
    oracle_fresnel, oracle_aces) bit for bit on random unit vectors, albedos, roughness and
    metalness, and on tone-mapping inputs from 0 to 100."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    (tmp_path / "main.cpp").write_text('#include "device_math.cuh"\n' + SHADE_MAIN)
    exe = tmp_path / "shade"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, str(tmp_path / "main.cpp"), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    rng = np.random.default_rng(9)
    n = 4000

    def unit(k):
        v = rng.standard_normal((k, 3))
        return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)

    rows = np.concatenate([unit(n), unit(n), unit(n), rng.uniform(0, 1, (n, 3)), rng.choice([0.0, 1.0], (n, 1)),
                           rng.uniform(0.0, 1.0, (n, 1)), rng.uniform(0.0, 1.0, (n, 1)), rng.uniform(-0.2, 1.2, (n, 1)),
                           rng.uniform(0.0, 1.0, (n, 1)), rng.uniform(0.0, 100.0, (n, 3)) ** rng.uniform(0.3, 1.0, (n, 1))],
                          axis=1).astype(np.float32)
    rows.tofile(tmp_path / "in.bin")
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    out = np.fromfile(tmp_path / "out.bin", np.float32).reshape(-1, 7)
    ref = np.array([oracle_py.brdf(rw[0:3], rw[3:6], rw[6:9], rw[9:12], rw[12], rw[13], rw[14])
                    + (oracle_py.fresnel(rw[15], rw[16]),) + oracle_py.aces(rw[17:20]) for rw in rows], np.float32)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), np.argwhere(out.view(np.uint32) != ref.view(np.uint32))[:5]


MARCH_MAIN = harness_source("march_rays.inc")


MARCH_SCENES = ["gallery", "spheres", "cornell", "csg_zoo", "unbounded_mix", "procedural3", "procedural8"]
SHADOW_SCENES = ["gallery", "spheres", "cornell", "procedural0", "procedural3", "procedural8", "procedural11"]


def _state_machine_exes(root, names, main):
    """Harnesses of the device march / shadow state machines with each scene's generated field."""
    jobs = {}
    for name in names:
        defines, ns = spec_namespace(SCENES[name]()[0])
        d = root / name
        d.mkdir()
        (d / "main.cpp").write_text(defines + '#include "march_kernels.cuh"\nnamespace mm3e { namespace spec {\n' + ns +
                                    "\n}}\n" + main)
        jobs[name] = (d, ["-include", SHIM, "-include", STUBS])
    return compile_harnesses(jobs, "harness")


@pytest.fixture(scope="module")
def march_exes(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    return _state_machine_exes(tmp_path_factory.mktemp("march"), MARCH_SCENES, MARCH_MAIN)


@pytest.mark.parametrize("name", MARCH_SCENES)
def test_march_state_machine_equals_oracle_on_host(name, march_exes, tmp_path):
    """The device march (march_kernels.cuh m_start / m_step: enhanced sphere tracing with its
    rollback, gap-cover and tetrahedral-normal phases, march.rs:120-223), compiled for the host and
    driven ray by ray over both the tape interpreter's field and the scene's generated field,
    against the oracle's march (oracle_march_rays): hit or miss, material, steps, and t and the
    normal of every hit, bit for bit, on rays from the scene's camera."""
    scene, cam = SCENES[name]()
    exe = march_exes[name]
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    n = 3000
    eye = np.array(cam.eye, np.float32)
    fwd, right, up = (np.array(v, np.float64) for v in (cam.forward, cam.right, cam.up))
    d = fwd + np.outer(rng.uniform(-1, 1, n) * cam.fov_scale * 1.7, right) + np.outer(rng.uniform(-1, 1, n) * cam.fov_scale, up)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays = np.concatenate([np.repeat(eye[None], n, 0), d], axis=1).astype(np.float32)
    (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    rays.tofile(tmp_path / "rays.bin")
    subprocess.run([str(exe), str(tmp_path / "tape.bin"), str(tmp_path / "rays.bin"), str(tmp_path / "out.bin")],
                   check=True)
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    per = n * 16 + n * 8
    ot, om, os_, on = oracle_py.march_rays(scene.desc(), rays, threads=2, normals=True)
    hit = om != 0xFFFFFFFF
    for k, label in enumerate(("interpreter", "specialised")):
        blk = raw[k * per:(k + 1) * per]
        hn = blk[:n * 16].view(np.float32).reshape(n, 4)
        hm = blk[n * 16:].view(np.uint32).reshape(n, 2)
        assert np.array_equal(hm[:, 0], om), label
        assert np.array_equal(hm[:, 1], os_), label
        assert np.array_equal(hn[hit, 3].view(np.uint32), ot[hit].astype(np.float32).view(np.uint32)), label
        assert np.array_equal(hn[hit, :3].view(np.uint32), on[hit].astype(np.float32).view(np.uint32)), label
    assert hit.mean() > 0.2


SHADOW_MAIN = harness_source("shadow_ao.inc")


@pytest.fixture(scope="module")
def shadow_exes(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    return _state_machine_exes(tmp_path_factory.mktemp("shadow"), SHADOW_SCENES, SHADOW_MAIN)


@pytest.mark.parametrize("name", SHADOW_SCENES)
def test_shadow_and_ao_equal_oracle_on_host(name, shadow_exes, tmp_path):
    """The device soft-shadow march (march_kernels.cuh s_start / s_step: the lifted origin, the
    light's direction, distance and k, the jittered start and the min(k h / t) fold with its
    division skip, march.rs:227-259 and lib.rs:1315-1333), compiled for the host and run over the
    device march's own hits with both the tape interpreter's field and the scene's generated field,
    against the oracle's soft shadow at its own hits (oracle_soft_shadows): every (ray, light)
    factor bit for bit, and -1 on the same pairs where no shadow ray is cast. The host sinf is the
    oracle's, so the jitter is bit-equal here; on the device it is within sinf's error bound.
    The AO pass (ao_slot, march.rs:264-280) runs over the same hits against oracle_ambient_occlusion,
    bit for bit, and leaves 1 on a miss."""
    scene, cam = SCENES[name]()
    nl = scene.desc().desc.n_lights
    assert nl > 0
    exe = shadow_exes[name]
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    n = 2000
    eye = np.array(cam.eye, np.float32)
    fwd, right, up = (np.array(v, np.float64) for v in (cam.forward, cam.right, cam.up))
    d = fwd + np.outer(rng.uniform(-1, 1, n) * cam.fov_scale * 1.7, right) + np.outer(rng.uniform(-1, 1, n) * cam.fov_scale, up)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays = np.concatenate([np.repeat(eye[None], n, 0), d], axis=1).astype(np.float32)
    (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    rays.tofile(tmp_path / "rays.bin")
    subprocess.run([str(exe), str(tmp_path / "tape.bin"), str(tmp_path / "rays.bin"), str(tmp_path / "out.bin"),
                    str(nl)], check=True)
    out = np.fromfile(tmp_path / "out.bin", np.float32).reshape(2, n * nl + n)
    ref = oracle_py.soft_shadows(scene.desc(), rays, threads=2)
    ref_occ = oracle_py.ambient_occlusion(scene.desc(), rays, threads=2)
    cast = ref >= 0
    lit = ref_occ >= 0
    assert lit.mean() > 0.2
    for k, label in enumerate(("interpreter", "specialised")):
        dev, occ = out[k, :n * nl].reshape(n, nl), out[k, n * nl:]
        assert np.array_equal(occ[lit].view(np.uint32), ref_occ[lit].view(np.uint32)), label
        assert np.array_equal(dev >= 0, cast), label
        assert np.array_equal(dev[cast].view(np.uint32), ref[cast].view(np.uint32)), \
            (label, np.argwhere(dev.view(np.uint32) != ref.view(np.uint32))[:5])
    assert cast.mean() > 0.1
    assert ((ref[cast] > 0) & (ref[cast] < 1)).any() and (ref[cast] == 0).any()
