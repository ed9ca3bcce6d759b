"""Scene-specialised fields against the tape interpreter, on the host.

The specialised program (spec_gen.cpp's generated field: inlined objects, generated CSG programs,
axis planes, linearised and enclosing-sphere pre-tests, weak bounds and skips) and the
interpreter's world_eval (WorldPlan::eval, accel.rs:209-252) compile as plain C++ with the host
definitions of the device intrinsics in tests/host_field/host_shim.h. Both are evaluated on the
same binary32 points over the scene's lowered tape (mm3e_scene_tape), and their (distance,
material) pairs must agree bit for bit. This covers many seeded scenes without a GPU; the GPU
tests check the same identity on the device (test_gpu_spec.py)."""
import os
import shutil
import subprocess
import zlib
from math import radians

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from mm3e_cuda import abi, scenes
from mm3e_cuda.scene import (GiVolume, Material, Object, Prim, Scene, SdfVolume, Transform, directional, look_at,
                             orbit_camera)
from field_scenes import csg_zoo_scene, noncons_scene, planes_scene, smooth_chain_scene, unbounded_mix_scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "atom-3d-engine_gb300", "csrc")
HOST_DIR = os.path.join(ROOT, "tests", "host_field")
SHIM = os.path.join(HOST_DIR, "host_shim.h")
CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")

MAIN = r"""
#include "host_io.h"
#include <cstdio>
#include <vector>
namespace mm3e { namespace spec {
#include "field.inc"
}}
using namespace mm3e;
int main(int argc, char** argv) {
    std::vector<float4> tape_words = read_words(argv[1]);
    const Tape T = tape_view(reinterpret_cast<const unsigned char*>(tape_words.data()));
    const std::vector<float> pts = read_floats(argv[2]);
    const size_t n = pts.size() / 3;
    size_t bad = 0;
    for (size_t k = 0; k < n; ++k) {
        V p{pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]};
        Field a = spec::eval(T, p), b = world_eval(T, p);
        const bool both_nan = a.d != a.d && b.d != b.d;
        if (!both_nan && (__float_as_uint(a.d) != __float_as_uint(b.d) || a.m != b.m)) {
            if (bad < 5) std::printf("mismatch at (%.9g, %.9g, %.9g): %.9g/%u vs %.9g/%u\n", p.x, p.y, p.z, a.d, a.m, b.d, b.m);
            bad += 1;
        }
    }
    std::printf("points %zu mismatches %zu\n", n, bad);
    return bad ? 1 : 0;
}
"""

SCENES = {
    "gallery": lambda: scenes.gallery_scene(64, 36),
    "spheres": lambda: scenes.spheres_scene(64, 36),
    "cornell": lambda: scenes.cornell_scene(64, 36),
    "planes": lambda: planes_scene(64, 36),
    "noncons": lambda: noncons_scene(21, 64, 36),
    "smooth_chain": lambda: smooth_chain_scene(5, 64, 36),
    "csg_zoo": lambda: csg_zoo_scene(2, 64, 36),
    "unbounded_mix": lambda: unbounded_mix_scene(4, 64, 36),
    **{f"procedural{k}": (lambda k=k: scenes.procedural_scene(k, 64, 36)) for k in (0, 3, 5, 8, 11, 12)},
}


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


@pytest.mark.parametrize("name", list(SCENES))
def test_specialised_field_equals_interpreter_on_host(name, tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    scene, cam = SCENES[name]()
    src = mm3e_cuda.spec_source(scene)
    body = src[src.index("namespace spec {") + len("namespace spec {"):src.index("struct Field_")]
    defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
    (tmp_path / "field.inc").write_text(body)
    (tmp_path / "main.cpp").write_text(defines + '#include "device_math.cuh"\n' + MAIN)
    exe = tmp_path / "field_check"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE, "-I", CSRC, "-I", HOST_DIR,
           "-I", str(tmp_path), "-include", SHIM, str(tmp_path / "main.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    _points(scene, cam, np.random.default_rng(zlib.crc32(name.encode()))).tofile(tmp_path / "points.bin")
    r = subprocess.run([str(exe), str(tmp_path / "tape.bin"), str(tmp_path / "points.bin")], capture_output=True,
                       text=True)
    print(name, r.stdout.strip().splitlines()[-1] if r.stdout.strip() else r.stderr[-500:])
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]


INTERP_MAIN = r"""
#include "host_io.h"
#include <cstdio>
#include <vector>
using namespace mm3e;
int main(int argc, char** argv) {
    std::vector<float4> tape_words = read_words(argv[1]);
    const Tape T = tape_view(reinterpret_cast<const unsigned char*>(tape_words.data()));
    const std::vector<float> pts = read_floats(argv[2]);
    const size_t n = pts.size() / 3;
    FILE* fo = std::fopen(argv[3], "wb");
    for (size_t k = 0; k < n; ++k) {
        Field f = world_eval(T, V{pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]});
        std::fwrite(&f.d, 4, 1, fo);
        std::fwrite(&f.m, 4, 1, fo);
    }
    std::fclose(fo);
    return 0;
}
"""


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


SHADE_MAIN = r"""
#include <cstdio>
#include <vector>
using namespace mm3e;
// per input row: n(3) l(3) v(3) albedo(3) metallic roughness reflectance cos f0 x(3) -> brdf(3) fresnel aces(3)
int main(int argc, char** argv) {
    FILE* fi = std::fopen(argv[1], "rb");
    std::vector<float> in(21 << 16);
    size_t n = std::fread(in.data(), sizeof(float), in.size(), fi) / 20;
    std::fclose(fi);
    FILE* fo = std::fopen(argv[2], "wb");
    for (size_t k = 0; k < n; ++k) {
        const float* r = &in[20 * k];
        V b = brdf(V{r[0], r[1], r[2]}, V{r[3], r[4], r[5]}, V{r[6], r[7], r[8]}, V{r[9], r[10], r[11]}, r[12], r[13], r[14]);
        float f = fresnel_schlick(r[15], r[16]);
        float a[3] = {aces1(r[17]), aces1(r[18]), aces1(r[19])};
        float o[7] = {b.x, b.y, b.z, f, a[0], a[1], a[2]};
        std::fwrite(o, sizeof(float), 7, fo);
    }
    std::fclose(fo);
    return 0;
}
"""


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


STUBS = os.path.join(HOST_DIR, "host_kernel_stubs.h")

MARCH_MAIN = r"""
#include "host_io.h"
#include <cstdio>
#include <vector>
using namespace mm3e;
using namespace mm3e::wave;
template <class FP> static void march_all(WaveArgs& a, const unsigned char* tape, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        MLane L;
        L.item = (uint32_t)i;
        L.phase = M_IDLE;
        LaneTape<TM_MULTI> LT;
        LT.p = tape;
        if (m_start<TM_MULTI, FP>(L, LT, a))
            while (L.phase != M_IDLE) m_step<TM_MULTI, FP>(L, LT, a);
    }
}
int main(int argc, char** argv) {
    std::vector<float4> tape_words = read_words(argv[1]);
    const unsigned char* tape = reinterpret_cast<const unsigned char*>(tape_words.data());
    const std::vector<float> rays = read_floats(argv[2]);
    const size_t n = rays.size() / 6;
    std::vector<float4> qo(n), qd(n), hn(n);
    std::vector<uint2> hm(n);
    for (size_t i = 0; i < n; ++i) {
        qo[i] = make_float4(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2], __uint_as_float((uint32_t)i));
        qd[i] = make_float4(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5], 0.0f);
    }
    WaveArgs a{};
    a.job0.tape = tape;
    a.src = SRC_QUEUE;
    a.b.q_o = qo.data();
    a.b.q_d = qd.data();
    a.b.h_n = hn.data();
    a.b.h_m = hm.data();
    FILE* fo = std::fopen(argv[3], "wb");
    march_all<InterpField>(a, tape, n);
    std::fwrite(hn.data(), sizeof(float4), n, fo);
    std::fwrite(hm.data(), sizeof(uint2), n, fo);
    march_all<spec::Field_>(a, tape, n);
    std::fwrite(hn.data(), sizeof(float4), n, fo);
    std::fwrite(hm.data(), sizeof(uint2), n, fo);
    std::fclose(fo);
    return 0;
}
"""


@pytest.mark.parametrize("name", ["gallery", "spheres", "cornell", "csg_zoo", "unbounded_mix", "procedural3", "procedural8"])
def test_march_state_machine_equals_oracle_on_host(name, tmp_path):
    """The device march (march_kernels.cuh m_start / m_step: enhanced sphere tracing with its
    rollback, gap-cover and tetrahedral-normal phases, march.rs:120-223), compiled for the host and
    driven ray by ray over both the tape interpreter's field and the scene's generated field,
    against the oracle's march (oracle_march_rays): hit or miss, material, steps, and t and the
    normal of every hit, bit for bit, on rays from the scene's camera."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    scene, cam = SCENES[name]()
    src = mm3e_cuda.spec_source(scene)
    ns = src[src.index("namespace spec {") + len("namespace spec {"):src.index("}  // namespace spec")]
    defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
    (tmp_path / "main.cpp").write_text(defines + '#include "march_kernels.cuh"\nnamespace mm3e { namespace spec {\n' + ns +
                                       "\n}}\n" + MARCH_MAIN)
    exe = tmp_path / "march"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS, str(tmp_path / "main.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
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


SHADOW_MAIN = r"""
#include "host_io.h"
#include <cstdio>
#include <vector>
using namespace mm3e;
using namespace mm3e::wave;
template <class FP> static void march_all(WaveArgs& a, const unsigned char* tape, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        MLane L;
        L.item = (uint32_t)i;
        L.phase = M_IDLE;
        LaneTape<TM_MULTI> LT;
        LT.p = tape;
        if (m_start<TM_MULTI, FP>(L, LT, a))
            while (L.phase != M_IDLE) m_step<TM_MULTI, FP>(L, LT, a);
    }
}
template <class FP> static void shadow_all(WaveArgs& a, const unsigned char* tape, size_t n) {
    // Items run light-major, as the persistent pass hands them out; s_start maps each to its slot.
    for (size_t i = 0; i < n * a.lights_max; ++i) {
        SLane S;
        S.item = (uint32_t)i;
        LaneTape<TM_MULTI> LT;
        LT.p = tape;
        if (s_start<TM_MULTI, FP>(S, LT, a, (uint32_t)n))
            while (S.item != NIL) s_step<TM_MULTI, FP>(S, LT, a);
    }
}
int main(int argc, char** argv) {
    std::vector<float4> tape_words = read_words(argv[1]);
    const unsigned char* tape = reinterpret_cast<const unsigned char*>(tape_words.data());
    const std::vector<float> rays = read_floats(argv[2]);
    const size_t n = rays.size() / 6;
    const uint32_t nl = (uint32_t)std::atoi(argv[4]);
    std::vector<float4> qo(n), qd(n), hn(n);
    std::vector<uint2> hm(n);
    std::vector<float> sh(n * nl), occ(n);
    for (size_t i = 0; i < n; ++i) {
        qo[i] = make_float4(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2], __uint_as_float((uint32_t)i));
        qd[i] = make_float4(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5], 0.0f);
    }
    WaveArgs a{};
    a.job0.tape = tape;
    a.src = SRC_QUEUE;
    a.lights_max = nl;
    a.b.q_o = qo.data();
    a.b.q_d = qd.data();
    a.b.h_n = hn.data();
    a.b.h_m = hm.data();
    a.b.shadow = sh.data();
    a.b.occ = occ.data();
    FILE* fo = std::fopen(argv[3], "wb");
    march_all<InterpField>(a, tape, n);
    shadow_all<InterpField>(a, tape, n);
    for (size_t i = 0; i < n; ++i) ao_slot<InterpField>(a, (uint32_t)i);
    std::fwrite(sh.data(), sizeof(float), sh.size(), fo);
    std::fwrite(occ.data(), sizeof(float), n, fo);
    march_all<spec::Field_>(a, tape, n);
    shadow_all<spec::Field_>(a, tape, n);
    for (size_t i = 0; i < n; ++i) ao_slot<spec::Field_>(a, (uint32_t)i);
    std::fwrite(sh.data(), sizeof(float), sh.size(), fo);
    std::fwrite(occ.data(), sizeof(float), n, fo);
    std::fclose(fo);
    return 0;
}
"""


@pytest.mark.parametrize("name", ["gallery", "spheres", "cornell", "procedural0", "procedural3", "procedural8", "procedural11"])
def test_shadow_and_ao_equal_oracle_on_host(name, tmp_path):
    """The device soft-shadow march (march_kernels.cuh s_start / s_step: the lifted origin, the
    light's direction, distance and k, the jittered start and the min(k h / t) fold with its
    division skip, march.rs:227-259 and lib.rs:1315-1333), compiled for the host and run over the
    device march's own hits with both the tape interpreter's field and the scene's generated field,
    against the oracle's soft shadow at its own hits (oracle_soft_shadows): every (ray, light)
    factor bit for bit, and -1 on the same pairs where no shadow ray is cast. The host sinf is the
    oracle's, so the jitter is bit-equal here; on the device it is within sinf's error bound.
    The AO pass (ao_slot, march.rs:264-280) runs over the same hits against oracle_ambient_occlusion,
    bit for bit, and leaves 1 on a miss."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    scene, cam = SCENES[name]()
    nl = scene.desc().desc.n_lights
    assert nl > 0
    src = mm3e_cuda.spec_source(scene)
    ns = src[src.index("namespace spec {") + len("namespace spec {"):src.index("}  // namespace spec")]
    defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
    (tmp_path / "main.cpp").write_text(defines + '#include <cstdlib>\n#include "march_kernels.cuh"\n'
                                       'namespace mm3e { namespace spec {\n' + ns + "\n}}\n" + SHADOW_MAIN)
    exe = tmp_path / "shadow"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS, str(tmp_path / "main.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
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


FRAME_MAIN = r"""
#include "host_io.h"
#include "host_passes.h"
#include <cstdio>
#include <cstdlib>
#include <vector>
using namespace mm3e;
using namespace mm3e::wave;
// One frame through the device pass sequence (host_passes.h), then the resolve of every pixel
// slot.
template <class FP>
static void frame(const unsigned char* tape, const CameraArgs& cam, uint32_t w, uint32_t h, uint32_t aa, float lens,
                  float focus, std::vector<float4>& hdr, std::vector<float4>& fg) {
    const uint32_t wlog = 3;
    const TapeHeader& H = *tape_view(tape).h;
    FrameJob J{};
    J.tape = tape;
    J.cam = cam;
    J.width = w;
    J.height = h;
    J.aa = aa;
    J.spp = aa * aa;
    J.tiles_x = (w + 7u) / 8u;
    J.n_slots = J.tiles_x * ((h + 3u) / 4u) * 32u;
    J.n_samples = J.n_slots * J.spp;
    J.n_pixels = w * h;
    J.n_lights = H.n_lights;
    const bool film = lens >= 0.0f;  // film.rs render_film: thin-lens samples, coverage, foreground
    J.lens_radius = film ? lens : 0.0f;
    J.focus_distance = focus;
    HostFrame F;
    F.init(J.n_samples, H.bounces + 1u, H.n_lights, J.n_pixels);
    WaveArgs a{};
    a.job0 = J;
    a.n_jobs = 1;
    a.tile_wlog = wlog;
    a.film = film ? 1u : 0u;
    host_levels<FP>(a, tape, SRC_SAMPLES, J.n_samples, F);
    for (uint32_t s = 0; s < J.n_slots; ++s) resolve_slot(a, s, 1u);
    hdr = F.hdr;
    fg = F.fg;
}
int main(int argc, char** argv) {
    std::vector<float4> tape_words = read_words(argv[1]);
    const unsigned char* tape = reinterpret_cast<const unsigned char*>(tape_words.data());
    const CameraArgs cam = read_camera(argv[2]);
    const uint32_t w = (uint32_t)std::atoi(argv[4]), h = (uint32_t)std::atoi(argv[5]), aa = (uint32_t)std::atoi(argv[6]);
    const float lens = std::strtof(argv[7], nullptr), focus = std::strtof(argv[8], nullptr);
    // Payloads the device reads by address (the GI probe cubes, each SDF volume's samples) are
    // not in the tape's bytes: point the header and the volume records at host copies.
    TapeHeader* H = reinterpret_cast<TapeHeader*>(tape_words.data());
    std::vector<std::vector<float4>> payloads;
    for (int k = 9; k < argc; ++k) payloads.push_back(read_words(argv[k]));
    size_t next = 0;
    if (H->gi_nx) H->gi_cubes = payloads.at(next++).data();
    DevVolume* vols = reinterpret_cast<DevVolume*>(reinterpret_cast<unsigned char*>(H) + H->off_volumes);
    for (uint32_t v = 0; v < H->n_volumes; ++v) vols[v].data = reinterpret_cast<const float*>(payloads.at(next++).data());
    std::vector<float4> hdr, fg;
    FILE* fo = std::fopen(argv[3], "wb");
    frame<InterpField>(tape, cam, w, h, aa, lens, focus, hdr, fg);
    std::fwrite(hdr.data(), sizeof(float4), hdr.size(), fo);
    std::fwrite(fg.data(), sizeof(float4), fg.size(), fo);
    frame<spec::Field_>(tape, cam, w, h, aa, lens, focus, hdr, fg);
    std::fwrite(hdr.data(), sizeof(float4), hdr.size(), fo);
    std::fwrite(fg.data(), sizeof(float4), fg.size(), fo);
    std::fclose(fo);
    return 0;
}
"""


def _cornell_gi_scene():
    """The Cornell room with a GI probe volume baked by the oracle (6x6x6 probes, 4 samples)."""
    scene, cam = scenes.cornell_scene(64, 36)
    mn, size, dims, cubes = oracle_py.bake_gi(scene.desc(), (6, 6, 6), 4)
    scene.gi = GiVolume(mn, size, dims, cubes)
    return scene, cam


def _volume_scene():
    """A UV sphere baked to an SDF volume by the oracle (resolution 24, padding 0.25), a second,
    scaled instance of the volume and a box, on a plane, under a soft sun."""
    s = Scene(64, 36)
    grey = s.material(Material.solid((0.8, 0.8, 0.8), roughness=0.5))
    red = s.material(Material.solid((0.85, 0.12, 0.10), roughness=0.4, metallic=0.3))
    pos, tri = scenes.uv_sphere_mesh(12, 18, 1.0)
    vid = s.volume(SdfVolume(*oracle_py.bake_mesh_sdf(pos, tri, 24, 0.25)))
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, grey))
    s.add(Object(Prim.volume(vid), Transform.at((-1.0, 1.0, 0.0)), red))
    s.add(Object(Prim.volume(vid), Transform((1.4, 0.7, 0.5), scale=0.7), grey))
    s.add(Object(Prim.box((0.4, 0.4, 0.4)), Transform.at((0.3, 0.4, -1.5)), red))
    sun = directional((0.45, 0.8, -0.4), (2.2, 2.1, 2.0)).soft(1.0 / 16.0)
    s.sun_dir = sun.vec
    s.light(sun)
    return s, look_at((0.0, 2.0, -6.0), (0.0, 0.8, 0.0), (0.0, 1.0, 0.0), radians(45.0))


def _no_ao_samples_scene():
    """The gallery with AO on but no AO samples: ambient_occlusion then returns 1 (march.rs:266)."""
    s, cam = scenes.gallery_scene(64, 36)
    s.marcher.ao_samples = 0
    return s, cam


def _shading_zoo_scene():
    """Every primitive kind, with materials at their edges (metallic 0 and 1, roughness 0 and 1,
    specular 0 and 1, reflectivity 1, emissive-only, checker, material ids past the table that
    wrap around), lit by a directional light, a point light, a sphere light, a light inside an
    object and a dim light far away, with a coloured sky and two reflection bounces."""
    from mm3e_cuda.scene import Light
    s = Scene(64, 36)
    s.bounces = 2
    s.aa = 1
    s.sky_ambient = (0.3, 0.35, 0.5)
    s.ambient = (0.03, 0.02, 0.01)
    s.sun_dir = (0.2, 0.9, -0.3)
    mats = [Material((0.8, 0.8, 0.8), roughness=0.0, metallic=1.0, reflectivity=1.0),
            Material((0.7, 0.2, 0.1), roughness=1.0, specular=0.0),
            Material((0.1, 0.6, 0.3), roughness=0.0, specular=1.0, metallic=0.0),
            Material((0.0, 0.0, 0.0), emissive=(3.0, 2.0, 0.5)),
            Material((0.9, 0.9, 0.9), checker=True, roughness=0.6),
            Material((0.2, 0.3, 0.9), metallic=0.5, roughness=0.02, reflectivity=0.4)]
    s.materials = list(mats)
    s.add(Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, 4))
    prims = [Prim.sphere(0.5), Prim.box((0.4, 0.3, 0.5)), Prim.round_box((0.3, 0.3, 0.3), 0.1),
             Prim.torus(0.4, 0.12), Prim.cylinder(0.4, 0.3), Prim.capsule((0.0, -0.3, 0.0), (0.0, 0.3, 0.0), 0.2),
             Prim.cone(0.4, 0.1, 0.5), Prim.ellipsoid((0.5, 0.3, 0.4)), Prim.octahedron(0.5), Prim.hex_prism(0.35, 0.3)]
    for k, pr in enumerate(prims):
        x, z = -3.0 + 1.5 * (k % 5), 1.0 + 1.6 * (k // 5)
        s.add(Object(pr, Transform((x, 0.6, z)), k % 6 if k < 6 else 6 + k))  # ids from 6 wrap around
    s.light(directional((0.4, 0.8, -0.5), (1.5, 1.4, 1.3)).soft(0.05))
    s.light(Light.point((1.0, 2.5, -1.0), (4.0, 3.0, 2.0)))
    s.light(Light.sphere((-2.0, 1.5, 0.5), (3.0, 3.0, 4.0), 0.3))
    s.light(Light.point((-3.0, 0.6, 1.0), (5.0, 5.0, 5.0)))  # inside the sphere at x = -3
    s.light(Light.point((40.0, 30.0, 60.0), (0.5, 0.5, 0.5)))
    return s, look_at((0.0, 3.0, -5.5), (0.0, 0.5, 1.5), (0.0, 1.0, 0.0), radians(55.0))


FRAME_SCENES = {**SCENES, "cornell_gi": _cornell_gi_scene, "volumes": _volume_scene,
                "no_ao_samples": _no_ao_samples_scene, "shading_zoo": _shading_zoo_scene}


def _build_frame_harness(scene, work):
    """Compile the frame harness with the scene's generated field into `work`; its path."""
    src = mm3e_cuda.spec_source(scene)
    ns = src[src.index("namespace spec {") + len("namespace spec {"):src.index("}  // namespace spec")]
    defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
    (work / "main.cpp").write_text(defines + '#include "shade_kernels.cuh"\nnamespace mm3e { namespace spec {\n' + ns +
                                   "\n}}\n" + FRAME_MAIN)
    exe = work / "frame"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS, str(work / "main.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run_frame_harness(exe, scene, cam, work, lens=-1.0, focus=1.0):
    """Run a built frame harness: (2, h, w, 4) HDR and (2, h, w, 4) foreground, for the
    interpreter's field and the generated one."""
    d = scene.desc().desc
    (work / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    np.array(list(cam.eye) + list(cam.forward) + list(cam.right) + list(cam.up) + [cam.fov_scale],
             np.float32).tofile(work / "cam.bin")
    payloads = []
    if scene.gi is not None:  # float4 per face, 6 faces per probe
        cubes = scene.gi.cubes.reshape(-1, 6, 3)
        payloads.append(np.concatenate([cubes, np.zeros(cubes.shape[:2] + (1,), np.float32)], axis=2))
    payloads += [v.data for v in scene.volumes]
    for k, arr in enumerate(payloads):
        np.ascontiguousarray(arr, np.float32).tofile(work / f"payload{k}.bin")
    w, h = d.width, d.height
    subprocess.run([str(exe), str(work / "tape.bin"), str(work / "cam.bin"), str(work / "out.bin"), str(w),
                    str(h), str(max(d.aa, 1)), repr(float(lens)), repr(float(focus))] +
                   [str(work / f"payload{k}.bin") for k in range(len(payloads))], check=True)
    out = np.fromfile(work / "out.bin", np.float32).reshape(2, 2, h, w, 4)
    return out[:, 0], out[:, 1]


FRAME_CASES = ["gallery", "spheres", "cornell", "cornell_gi", "volumes", "no_ao_samples", "shading_zoo", "noncons",
               "smooth_chain",
               "csg_zoo", "unbounded_mix", "procedural0", "procedural3", "procedural8", "procedural11"]
FILM_CASES = [("gallery", 3, 0.08, 6.0), ("spheres", 2, 0.15, 5.0), ("csg_zoo", 2, 0.0, 1.0), ("cornell_gi", 1, 0.1, 4.0),
              ("procedural3", 2, 0.05, 8.0)]


def _film_scene(name, aa):
    scene, cam = FRAME_SCENES[name]()
    scene.aa = aa
    return scene, cam


@pytest.fixture(scope="module")
def frame_harnesses(tmp_path_factory):
    """Frame harnesses of every whole-frame and film case, compiled in parallel, by generated
    source (the same source builds once)."""
    from concurrent.futures import ThreadPoolExecutor
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    scenes_ = [FRAME_SCENES[n]()[0] for n in FRAME_CASES] + [_film_scene(n, aa)[0] for n, aa, _, _ in FILM_CASES]
    by_src = {}
    for sc in scenes_:
        by_src.setdefault(mm3e_cuda.spec_source(sc), sc)
    root = tmp_path_factory.mktemp("frame_harness")
    works = []
    for k in range(len(by_src)):
        (root / str(k)).mkdir()
        works.append(root / str(k))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        exes = list(pool.map(_build_frame_harness, by_src.values(), works))
    return dict(zip(by_src, exes))


@pytest.mark.parametrize("name", FRAME_CASES)
def test_frame_equals_oracle_render_on_host(name, frame_harnesses, tmp_path):
    """A whole frame through the device pass sequence (march_kernels.cuh and shade_kernels.cuh:
    camera samples, march, reflection queue, AO, soft shadows, shade_hit, the reflection fold and
    the AA average; lib.rs:1223-1360), compiled for the host and run pass by pass over both the
    tape interpreter's field and the scene's generated field, against the oracle's render
    (oracle_render's HDR radiance, before post): every pixel bit for bit. The scenes cover
    reflections, 2x2 AA, fog, checker albedo, lights and their shadows, and CSG. On the device
    only CUDA's transcendental functions (sinf, expf, powf, ...) differ from these."""
    scene, cam = FRAME_SCENES[name]()
    d = scene.desc().desc
    w, h = d.width, d.height
    out, _ = _run_frame_harness(frame_harnesses[mm3e_cuda.spec_source(scene)], scene, cam, tmp_path)
    _, ref = oracle_py.render(scene.desc(), cam, threads=2, want_hdr=True)
    assert ref.std() > 0.1 and len(np.unique(ref.reshape(-1, 3), axis=0)) > w * h // 2
    for k, label in enumerate(("interpreter", "specialised")):
        dev = np.ascontiguousarray(out[k, :, :, :3])
        bad = np.argwhere((dev.view(np.uint32) != ref.view(np.uint32)).any(axis=2))
        assert len(bad) == 0, (label, len(bad), [(tuple(p), dev[tuple(p)].tolist(), ref[tuple(p)].tolist())
                                                 for p in bad[:3]])


@pytest.mark.parametrize("name,aa,lens,focus", FILM_CASES)
def test_film_equals_oracle_on_host(name, aa, lens, focus, frame_harnesses, tmp_path):
    """render_film's samples (film.rs:147-196: the thin-lens ray of each AA sample through the
    aperture grid, camera.rs:71-102; coverage and the premultiplied foreground of primary hits)
    through the device pass sequence (march_kernels.cuh lens_ray, shade_kernels.cuh resolve_slot
    in film mode), compiled for the host, against the oracle's render_film: beauty, alpha and
    foreground bit for bit, for both fields. The cases cover a 3x3 and 2x2 aperture grid, a
    pinhole with AA, and a lens at one sample (the centre ray)."""
    scene, cam = _film_scene(name, aa)
    hdr, fg = _run_frame_harness(frame_harnesses[mm3e_cuda.spec_source(scene)], scene, cam, tmp_path, lens, focus)
    ref = oracle_py.render_film(scene.desc(), cam, lens, focus, threads=2)
    assert 0.0 < ref["alpha"].mean() < 1.0 and ref["beauty"].std() > 0.1
    for k, label in enumerate(("interpreter", "specialised")):
        for got, want, what in ((hdr[k, :, :, :3], ref["beauty"], "beauty"), (hdr[k, :, :, 3], ref["alpha"], "alpha"),
                                (fg[k, :, :, :3], ref["foreground"], "foreground")):
            got = np.ascontiguousarray(got)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
                (label, what, int((got.view(np.uint32) != want.view(np.uint32)).sum()))


GI_MAIN = r"""
#include <cstring>
#include <vector>
#include "lower.h"
using namespace mm3e;
using namespace mm3e::wave;
// The device GI bake (mm3e_bake_gi) pass by pass: the product's probe grid and gather directions
// (gi_setup), the SRC_GATHER march of every (probe, face, direction) ray, the gather shading of
// its hit, and the per-face weighted average. Cubes out as (probe, face, rgb).
template <class FP>
static void bake(const GiSetup& g, const unsigned char* tape, float* cubes18) {
    const uint64_t probes = (uint64_t)g.nx * g.ny * g.nz, items = probes * 6u * g.dirs_per_face;
    std::vector<float4> q_o(items), q_d(items), h_n(items), rad(items), dirs(g.dirs.size() / 4), cubes(probes * 6u);
    std::vector<uint2> h_m(items);
    std::memcpy(dirs.data(), g.dirs.data(), g.dirs.size() * sizeof(float));
    WaveArgs a{};
    a.job0.tape = tape;
    a.src = SRC_GATHER;
    a.n_items = (uint32_t)items;
    a.cap = (uint32_t)items;
    a.b.q_o = q_o.data();
    a.b.q_d = q_d.data();
    a.b.h_n = h_n.data();
    a.b.h_m = h_m.data();
    std::memcpy(a.gi_lo, g.lo, 12);
    std::memcpy(a.gi_cell, g.cell, 12);
    a.gi_nx = g.nx;
    a.gi_ny = g.ny;
    a.gi_nz = g.nz;
    a.dirs_per_face = g.dirs_per_face;
    a.gather_dirs = dirs.data();
    for (uint64_t i = 0; i < items; ++i) {
        MLane L;
        L.item = (uint32_t)i;
        L.phase = M_IDLE;
        LaneTape<TM_MULTI> LT;
        LT.p = tape;
        if (m_start<TM_MULTI, FP>(L, LT, a))
            while (L.phase != M_IDLE) m_step<TM_MULTI, FP>(L, LT, a);
    }
    for (uint64_t i = 0; i < items; ++i) gather_slot(a, (uint32_t)i, rad.data());
    for (uint64_t i = 0; i < probes * 6u; ++i) gi_reduce_slot(rad.data(), dirs.data(), g.dirs_per_face, (uint32_t)i, cubes.data());
    for (uint64_t i = 0; i < probes * 6u; ++i) {
        cubes18[3 * i] = cubes[i].x;
        cubes18[3 * i + 1] = cubes[i].y;
        cubes18[3 * i + 2] = cubes[i].z;
    }
}
extern "C" int host_bake_gi(const mm3e_scene_desc* d, const unsigned char* tape_bytes, size_t tape_len, uint32_t nx,
                            uint32_t ny, uint32_t nz, uint32_t samples, int specialised, float* lo_size6,
                            uint32_t* dims3, float* cubes18) {
    GiSetup g;
    if (!gi_setup(*d, nx, ny, nz, samples, g)) return 0;
    std::vector<float4> words((tape_len + 15) / 16);
    std::memcpy(words.data(), tape_bytes, tape_len);
    const unsigned char* tape = reinterpret_cast<const unsigned char*>(words.data());
    std::memcpy(lo_size6, g.lo, 12);
    std::memcpy(lo_size6 + 3, g.size, 12);
    dims3[0] = g.nx;
    dims3[1] = g.ny;
    dims3[2] = g.nz;
    if (specialised) bake<spec::Field_>(g, tape, cubes18);
    else bake<InterpField>(g, tape, cubes18);
    return 1;
}
"""


@pytest.mark.parametrize("name,dims,samples", [("cornell", (6, 5, 4), 5), ("gallery", (5, 4, 5), 5),
                                               ("spheres", (4, 4, 4), 1), ("procedural8", (4, 3, 4), 5)])
def test_gi_bake_equals_oracle_on_host(name, dims, samples, tmp_path):
    """The device GI bake (mm3e_bake_gi: gi_setup's probe grid and directions, lower.cpp; the
    SRC_GATHER march, march_kernels.cuh; gather_slot and gi_reduce_slot, shade_kernels.cuh;
    Scene::bake_gi_unchecked, lib.rs:668-711, gi.rs:38-125), compiled for the host with the
    product's own set-up code and run over both the interpreter's field and the generated one,
    against the oracle's bake_gi on the same descriptor: grid bounds, dims and every cube face
    bit for bit. On the device only CUDA's transcendental functions differ."""
    import ctypes as C
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    scene, _ = SCENES[name]()
    src = mm3e_cuda.spec_source(scene)
    ns = src[src.index("namespace spec {") + len("namespace spec {"):src.index("}  // namespace spec")]
    defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
    (tmp_path / "main.cpp").write_text(defines + '#include "shade_kernels.cuh"\nnamespace mm3e { namespace spec {\n' + ns +
                                       "\n}}\n" + GI_MAIN)
    lib_path = tmp_path / "libhostgi.so"
    flags = ["-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-fPIC", "-I", CUDA_INCLUDE, "-I", CSRC, "-I", HOST_DIR]
    r = subprocess.run(["g++"] + flags + ["-c", os.path.join(CSRC, "lower.cpp"), "-o", str(tmp_path / "lower.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run(["g++"] + flags + ["-include", SHIM, "-include", STUBS, "-shared", str(tmp_path / "main.cpp"),
                                          str(tmp_path / "lower.o"), "-o", str(lib_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = C.CDLL(str(lib_path))
    handle = scene.desc()
    tape = mm3e_cuda.scene_tape(scene)
    mn, size, rdims, ref = oracle_py.bake_gi(handle, dims, samples)
    n = rdims[0] * rdims[1] * rdims[2]
    for specialised in (0, 1):
        lo_size = np.zeros(6, np.float32)
        got_dims = np.zeros(3, np.uint32)
        cubes = np.zeros(n * 18, np.float32)
        ok = lib.host_bake_gi(C.c_void_p(C.addressof(handle.desc)), tape, C.c_size_t(len(tape)), *[C.c_uint32(v) for v in dims],
                              C.c_uint32(samples), C.c_int(specialised), lo_size.ctypes.data_as(C.c_void_p),
                              got_dims.ctypes.data_as(C.c_void_p), cubes.ctypes.data_as(C.c_void_p))
        assert ok == 1
        assert tuple(got_dims) == tuple(rdims)
        assert np.array_equal(lo_size.view(np.uint32), np.array(list(mn) + list(size), np.float32).view(np.uint32))
        assert np.array_equal(cubes.view(np.uint32), ref.view(np.uint32)), \
            (specialised, int((cubes.view(np.uint32) != ref.view(np.uint32)).sum()), n * 18)
    assert ref.std() > 0.01


AOV_MAIN = r"""
#include "host_io.h"
using namespace mm3e;
using namespace mm3e::wave;
// An AOV frame as the device runs it: the pixel-centre march (SRC_CENTER), the AO pass in the AO
// mode, and the display value of every pixel.
template <class FP> static void aov(const unsigned char* tape, const CameraArgs& cam, uint32_t w, uint32_t h,
                                    uint32_t mode, std::vector<float4>& out) {
    const uint32_t n = w * h;
    std::vector<float4> q_o(n), q_d(n), h_n(n);
    std::vector<uint2> h_m(n);
    std::vector<float> occ(n, -7.0f);
    out.assign(n, make_float4(0.f, 0.f, 0.f, 0.f));
    WaveArgs a{};
    a.job0.tape = tape;
    a.job0.cam = cam;
    a.job0.width = w;
    a.job0.height = h;
    a.src = SRC_CENTER;
    a.n_items = n;
    a.cap = n;
    a.aov_mode = mode;
    a.b.q_o = q_o.data();
    a.b.q_d = q_d.data();
    a.b.h_n = h_n.data();
    a.b.h_m = h_m.data();
    a.b.occ = occ.data();
    for (uint32_t i = 0; i < n; ++i) {
        MLane L;
        L.item = i;
        L.phase = M_IDLE;
        LaneTape<TM_MULTI> LT;
        LT.p = tape;
        if (m_start<TM_MULTI, FP>(L, LT, a))
            while (L.phase != M_IDLE) m_step<TM_MULTI, FP>(L, LT, a);
    }
    if (mode == MM3E_MODE_AO)
        for (uint32_t i = 0; i < n; ++i) ao_slot<FP>(a, i);
    for (uint32_t i = 0; i < n; ++i) aov_slot(a, i, out.data());
}
int main(int argc, char** argv) {
    std::vector<float4> tape_words = read_words(argv[1]);
    const unsigned char* tape = reinterpret_cast<const unsigned char*>(tape_words.data());
    const CameraArgs cam = read_camera(argv[2]);
    const uint32_t w = (uint32_t)std::atoi(argv[4]), h = (uint32_t)std::atoi(argv[5]), mode = (uint32_t)std::atoi(argv[6]);
    std::vector<float4> out;
    FILE* fo = std::fopen(argv[3], "wb");
    aov<InterpField>(tape, cam, w, h, mode, out);
    std::fwrite(out.data(), sizeof(float4), out.size(), fo);
    aov<spec::Field_>(tape, cam, w, h, mode, out);
    std::fwrite(out.data(), sizeof(float4), out.size(), fo);
    std::fclose(fo);
    return 0;
}
"""


@pytest.mark.parametrize("name", ["gallery", "csg_zoo", "procedural8"])
def test_aov_modes_equal_oracle_on_host(name, tmp_path):
    """The AOV display modes (lib.rs:1178-1218: normal, depth, AO, step heat map, albedo) as the
    device computes them (the SRC_CENTER march, the AO pass, shade_kernels.cuh aov_slot), compiled
    for the host, against the oracle's render in each mode: every pixel bit for bit, for both
    fields, and in the AO mode also with no AO samples (a white frame)."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    base, cam = FRAME_SCENES[name]()
    cases = [(m, None) for m in (abi.MODE_NORMAL, abi.MODE_DEPTH, abi.MODE_AO, abi.MODE_STEPS, abi.MODE_ALBEDO)]
    cases.append((abi.MODE_AO, 0))
    np.array(list(cam.eye) + list(cam.forward) + list(cam.right) + list(cam.up) + [cam.fov_scale],
             np.float32).tofile(tmp_path / "cam.bin")
    exes = {}  # by generated source: it bakes the marcher's settings (AO samples among them), not the mode
    for mode, ao_samples in cases:
        scene = base.copy()
        scene.mode = mode
        if ao_samples is not None:
            scene.marcher.ao_samples = ao_samples
        src = mm3e_cuda.spec_source(scene)
        if src not in exes:
            ns = src[src.index("namespace spec {") + len("namespace spec {"):src.index("}  // namespace spec")]
            defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
            k = len(exes)
            (tmp_path / f"main{k}.cpp").write_text(defines + '#include "shade_kernels.cuh"\nnamespace mm3e { namespace spec {\n' +
                                                   ns + "\n}}\n" + AOV_MAIN)
            exes[src] = tmp_path / f"aov{k}"
            r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I",
                                CUDA_INCLUDE, "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS,
                                str(tmp_path / f"main{k}.cpp"), "-o", str(exes[src])], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr[-3000:]
        exe = exes[src]
        (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
        d = scene.desc().desc
        w, h = d.width, d.height
        subprocess.run([str(exe), str(tmp_path / "tape.bin"), str(tmp_path / "cam.bin"), str(tmp_path / "out.bin"),
                        str(w), str(h), str(mode)], check=True)
        out = np.fromfile(tmp_path / "out.bin", np.float32).reshape(2, h, w, 4)
        ref = oracle_py.render(scene.desc(), cam)
        if ao_samples == 0:
            assert np.array_equal(ref, np.ones_like(ref))
        else:
            assert ref[..., :3].std() > 0.01, mode
        for k, label in enumerate(("interpreter", "specialised")):
            assert np.array_equal(out[k].view(np.uint32), ref.view(np.uint32)), \
                (label, mode, int((out[k].view(np.uint32) != ref.view(np.uint32)).any(axis=2).sum()))


SCENE_EDGES = {  # Scene / Marcher settings at their edges, each applied to the 48x27 gallery
    "aa0": {"aa": 0},
    "aa4": {"aa": 4},
    "steps0": {"max_steps": 0},
    "steps1": {"max_steps": 1},
    "steps7": {"max_steps": 7},
    "shadow_steps0": {"shadow_steps": 0},
    "shadow_steps1": {"shadow_steps": 1},
    "ao1": {"ao_samples": 1},
    "ao2": {"ao_samples": 2},
    "near_far": {"max_dist": 3.0},
    "eps0": {"eps": 0.0},
    "eps_big": {"eps": 0.05},
    "relaxed": {"step_scale": 0.6},
    "over_relaxed": {"step_scale": 1.6},
    "lod": {"lod_footprint": 0.002},
    "secant": {"secant": True},
    "subitize": {"subitize": 0.5},
    "secant_subitize_over": {"secant": True, "subitize": 0.3, "step_scale": 1.3},
    "normal_h0": {"normal_h": 0.0},
    "normal_h_big": {"normal_h": 0.05},
    "bounces3": {"bounces": 3},
    "bounces0": {"bounces": 0},
    "no_shadows_no_ao": {"shadows": False, "ao": False},
    "no_fog": {"fog_density": 0.0},
}


def test_frame_at_setting_edges_equals_oracle_on_host(tmp_path):
    """Whole frames at the edges of the scene's and the marcher's settings (AA 0 and 4, no or one
    march step, no shadow steps, one or two AO samples, a near far plane, zero and large epsilon,
    relaxed and over-relaxed steps, LOD, secant and subitize boosts, zero normal offsets, 0 and 3
    bounces, shadows, AO and fog off), through the device pass sequence over both fields, against
    the oracle's render bit for bit. The generated field folds these settings into constants, so
    this also checks every folded form against the interpreter's reading of the header. The
    harnesses compile in parallel."""
    from concurrent.futures import ThreadPoolExecutor
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    cases = {}
    for edge, settings in SCENE_EDGES.items():
        scene, cam = scenes.gallery_scene(48, 27)
        for key, value in settings.items():
            setattr(scene if hasattr(scene, key) else scene.marcher, key, value)
        work = tmp_path / edge
        work.mkdir()
        cases[edge] = (scene, cam, work)
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        exes = dict(zip(cases, pool.map(lambda c: _build_frame_harness(c[0], c[2]), cases.values())))
    failed = {}
    for edge, (scene, cam, work) in cases.items():
        out, _ = _run_frame_harness(exes[edge], scene, cam, work)
        _, ref = oracle_py.render(scene.desc(), cam, threads=2, want_hdr=True)
        for k, label in enumerate(("interpreter", "specialised")):
            dev = np.ascontiguousarray(out[k, :, :, :3])
            bad = int((dev.view(np.uint32) != ref.view(np.uint32)).any(axis=2).sum())
            if bad:
                failed[(edge, label)] = bad
    assert not failed, failed


PREVIEW_MAIN = r"""
#include "host_io.h"
#include "host_passes.h"
using namespace mm3e;
using namespace mm3e::wave;
using namespace mm3e::preview;
// The preview path as the device runs it (mm3e_render_gbuffer, mm3e_reproject): an aa-1 frame
// without post packed into a G-buffer with its primary hits and the movers' tags; the forward
// warp of that G-buffer into the new camera; the cheap row fill; and the hybrid re-render of the
// warp's holes through the pass sequence (the holes' rays as the primary level's queue) and
// their resolve. The kernels run as one thread of one block: each grid-stride loop visits every
// item in order, and the row fill (one thread per row) runs row by row.
template <class FP>
static void run_preview(const unsigned char* tape, const CameraArgs& c0, const CameraArgs& c1, uint32_t w, uint32_t h,
                    const std::vector<float>& movers, const std::vector<float>& deltas, FILE* fo) {
    const uint32_t wlog = 3, n = w * h;
    const TapeHeader& H = *tape_view(tape).h;
    FrameJob J{};
    J.tape = tape;
    J.cam = c0;
    J.width = w;
    J.height = h;
    J.aa = 1;
    J.spp = 1;
    J.tiles_x = (w + 7u) / 8u;
    J.n_slots = J.tiles_x * ((h + 3u) / 4u) * 32u;
    J.n_samples = J.n_slots;
    J.n_pixels = n;
    J.n_lights = H.n_lights;
    HostFrame F;
    F.init(J.n_samples, H.bounces + 1u, H.n_lights, n);
    WaveArgs a{};
    a.job0 = J;
    a.n_jobs = 1;
    a.tile_wlog = wlog;
    host_levels<FP>(a, tape, SRC_SAMPLES, J.n_samples, F);
    for (uint32_t s = 0; s < J.n_slots; ++s) resolve_slot(a, s, 1u);
    std::vector<uchar4> color(n);
    std::vector<float> depth(n);
    std::vector<int32_t> obj(n);
    k_gbuffer_pack(a, J.n_slots, reinterpret_cast<const float4*>(movers.data()), (uint32_t)(movers.size() / 4),
                   color.data(), depth.data(), obj.data());
    std::fwrite(color.data(), sizeof(uchar4), n, fo);
    std::fwrite(depth.data(), sizeof(float), n, fo);
    std::fwrite(obj.data(), sizeof(int32_t), n, fo);
    // forward warp, then the cheap fill
    std::vector<unsigned long long> keys(n, ~0ull);
    std::vector<uchar4> warped(n), cheap(n);
    std::vector<unsigned char> filled(n), cheap_filled(n);
    k_warp_keys(c0, c1, w, h, depth.data(), obj.data(), deltas.data(), (uint32_t)(deltas.size() / 3), keys.data());
    k_warp_apply(n, keys.data(), color.data(), warped.data(), filled.data());
    cheap = warped;
    cheap_filled = filled;
    for (uint32_t y = 0; y < h; ++y) {
        blockIdx.x = y;
        k_row_fill(w, h, cheap.data(), cheap_filled.data());
    }
    blockIdx.x = 0;
    std::fwrite(cheap.data(), sizeof(uchar4), n, fo);
    // hybrid: the holes' rays through the pass sequence, then their resolve into the warped frame
    HostFrame G;
    G.init(n, H.bounces + 1u, H.n_lights, n);
    std::vector<uint32_t> hole_pix(n);
    uint32_t count = 0;
    k_hole_rays(c1, w, h, filled.data(), G.q_o[0].data(), G.q_d[0].data(), hole_pix.data(), &count);
    WaveArgs b{};
    b.job0 = J;
    b.job0.cam = c1;
    b.n_jobs = 1;
    b.tile_wlog = wlog;
    host_levels<FP>(b, tape, SRC_QUEUE, count, G);
    b.n_items = n;
    std::vector<uchar4> hybrid = warped;
    k_hole_resolve(b, &count, hole_pix.data(), hybrid.data());
    std::fwrite(hybrid.data(), sizeof(uchar4), n, fo);
}
int main(int argc, char** argv) {
    blockDim.x = 1;
    gridDim.x = 1;
    std::vector<float4> tape_words = read_words(argv[1]);
    const unsigned char* tape = reinterpret_cast<const unsigned char*>(tape_words.data());
    const CameraArgs c0 = read_camera(argv[2]), c1 = read_camera(argv[3]);
    const uint32_t w = (uint32_t)std::atoi(argv[5]), h = (uint32_t)std::atoi(argv[6]);
    const std::vector<float> movers = read_floats(argv[7]), deltas = read_floats(argv[8]);
    FILE* fo = std::fopen(argv[4], "wb");
    run_preview<InterpField>(tape, c0, c1, w, h, movers, deltas, fo);
    run_preview<spec::Field_>(tape, c0, c1, w, h, movers, deltas, fo);
    std::fclose(fo);
    return 0;
}
"""


def _cam_bin(cam, path):
    np.array(list(cam.eye) + list(cam.forward) + list(cam.right) + list(cam.up) + [cam.fov_scale],
             np.float32).tofile(path)


PREVIEW_CASES = {  # scene, movers (x, y, z, radius), per-mover deltas
    "demo": (lambda: scenes.demo_scene(), [(-1.2, 1.0, 0.0, 1.3), (1.2, 0.6, 0.0, 0.8)], [(0.3, -0.2, 0.1), (0.0, 0.4, 0.0)]),
    "spheres": (lambda: scenes.spheres_scene(64, 36), [(0.0, 1.0, 0.0, 1.0), (-2.2, 1.0, 0.0, 1.0)], [(1.5, 0.0, 0.0)]),
    "gallery": (lambda: scenes.gallery_scene(64, 36), [], []),
    "hero_aa2_b2": (lambda: scenes.hero_scene(48, 27, 2, 2), [(0.0, 1.0, 0.0, 1.0)], [(0.0, 0.0, 0.0)]),
}


@pytest.mark.parametrize("name", list(PREVIEW_CASES))
def test_preview_path_equals_oracle_on_host(name, tmp_path):
    """The preview path (reproject_kernels.cuh: k_gbuffer_pack, k_warp_keys / k_warp_apply,
    k_row_fill, k_hole_rays, k_hole_resolve; lib.rs:951-1080, reproject.rs:55-146) with the
    pass sequence of host_passes.h, compiled for the host over both fields, against the oracle's
    render_gbuffer, reproject and reproject_hybrid: the G-buffer's colour, depth and object tags,
    the cheap reprojection and the hybrid frame, all bit for bit."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    make, movers, deltas = PREVIEW_CASES[name]
    scene, _ = make()
    c0 = orbit_camera((0.0, 0.8, 0.3), 7.0, 0.5, 0.3, radians(52.0))
    c1 = orbit_camera((0.0, 0.8, 0.3), 7.0, 0.62, 0.3, radians(52.0))
    src = mm3e_cuda.spec_source(scene)
    ns = src[src.index("namespace spec {") + len("namespace spec {"):src.index("}  // namespace spec")]
    defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
    (tmp_path / "main.cpp").write_text(defines + '#include "shade_kernels.cuh"\n#include "reproject_kernels.cuh"\n'
                                       'namespace mm3e { namespace spec {\n' + ns + "\n}}\n" + PREVIEW_MAIN)
    exe = tmp_path / "preview"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS, str(tmp_path / "main.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    _cam_bin(c0, tmp_path / "c0.bin")
    _cam_bin(c1, tmp_path / "c1.bin")
    np.array(movers, np.float32).reshape(-1).tofile(tmp_path / "movers.bin")
    np.array(deltas, np.float32).reshape(-1).tofile(tmp_path / "deltas.bin")
    d = scene.desc().desc
    w, h = d.width, d.height
    subprocess.run([str(exe), str(tmp_path / "tape.bin"), str(tmp_path / "c0.bin"), str(tmp_path / "c1.bin"),
                    str(tmp_path / "out.bin"), str(w), str(h), str(tmp_path / "movers.bin"), str(tmp_path / "deltas.bin")],
                   check=True)
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    n = w * h
    per = n * 4 * 3 + n * 4 * 2
    g = oracle_py.render_gbuffer(scene.desc(), c0, movers=movers)
    cheap = oracle_py.reproject(g, c0, c1, deltas)
    hybrid = oracle_py.reproject(g, c0, c1, deltas, hybrid_handle=scene.desc())
    holes = ~oracle_py.reproject_filled(g, c0, c1, deltas).astype(bool)
    assert holes.any() and (~holes).any()
    assert np.isfinite(g["depth"]).any() and (movers == [] or (g["obj"] >= 0).any())
    for k, label in enumerate(("interpreter", "specialised")):
        blk = raw[k * per:(k + 1) * per]
        color = blk[:n * 4].reshape(h, w, 4)
        depth = blk[n * 4:n * 8].view(np.float32).reshape(h, w)
        obj = blk[n * 8:n * 12].view(np.int32).reshape(h, w)
        got_cheap = blk[n * 12:n * 16].reshape(h, w, 4)
        got_hybrid = blk[n * 16:n * 20].reshape(h, w, 4)
        assert np.array_equal(color, g["color"]), (label, "colour", int((color != g["color"]).any(-1).sum()))
        assert np.array_equal(depth.view(np.uint32), g["depth"].view(np.uint32)), (label, "depth")
        assert np.array_equal(obj, g["obj"]), (label, "objects")
        assert np.array_equal(got_cheap, cheap), (label, "cheap", int((got_cheap != cheap).any(-1).sum()))
        assert np.array_equal(got_hybrid, hybrid), (label, "hybrid", int((got_hybrid != hybrid).any(-1).sum()))


def _random_case(rng):
    """A seeded random scene (procedural, CSG zoo, unbounded mix, non-conservative, smooth chain,
    gallery or hero), random scene and marcher settings, and a random orbit camera."""
    kind = rng.choice(["proc", "proc", "csg", "unb", "nc", "sc", "gallery", "hero"])
    w, h = rng.choice([(40, 24), (33, 17), (48, 27)])
    if kind == "proc":
        s, cam = scenes.procedural_scene(rng.randrange(1000), w, h)
    elif kind == "csg":
        s, cam = csg_zoo_scene(rng.randrange(50), w, h)
    elif kind == "unb":
        s, cam = unbounded_mix_scene(rng.randrange(50), w, h)
    elif kind == "nc":
        s, cam = noncons_scene(rng.randrange(50), w, h)
    elif kind == "sc":
        s, cam = smooth_chain_scene(rng.randrange(2, 9), w, h)
    elif kind == "gallery":
        s, cam = scenes.gallery_scene(w, h)
    else:
        s, cam = scenes.hero_scene(w, h, 2, 2)
    choices = {"aa": [1, 2, 3], "bounces": [0, 1, 2, 3], "step_scale": [0.5, 0.8, 1.0, 1.2, 1.6],
               "secant": [False, True], "subitize": [0.0, 0.2, 0.6], "lod_footprint": [0.0, 0.001, 0.006],
               "eps": [0.0, 0.0001, 0.002, 0.02], "max_steps": [8, 32, 96, 256], "shadow_steps": [0, 3, 16, 96],
               "ao_samples": [0, 1, 2, 8], "normal_h": [0.0, 0.0002, 0.01], "max_dist": [5.0, 30.0, 500.0],
               "fog_density": [0.0, 0.05, 0.3], "shadows": [False, True], "ao": [False, True]}
    settings = {k: rng.choice(v) for k, v in choices.items() if rng.random() < 0.35}
    for key, value in settings.items():
        setattr(s if hasattr(s, key) else s.marcher, key, value)
    if rng.random() < 0.5:
        cam = orbit_camera((rng.uniform(-1, 1), rng.uniform(0, 1.5), rng.uniform(-1, 1)), rng.uniform(2.0, 12.0),
                           rng.uniform(-3.1, 3.1), rng.uniform(-0.4, 1.2), radians(rng.uniform(25, 80)))
    return kind, settings, s, cam


def test_random_configurations_equal_oracle_on_host(tmp_path):
    """Eight seeded random configurations (scene kind, scene and marcher settings, camera), whole
    frames through the device pass sequence over both fields against the oracle's render, bit for
    bit; the odd ones also in film mode with a random thin lens against render_film."""
    import random
    from concurrent.futures import ThreadPoolExecutor
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    cases = []
    for k in range(8):
        rng = random.Random(20261204 + k)
        kind, settings, s, cam = _random_case(rng)
        lens, focus = (rng.choice([0.02, 0.1, 0.4]), rng.choice([0.5, 3.0, 7.0, 20.0])) if k % 2 else (-1.0, 1.0)
        work = tmp_path / str(k)
        work.mkdir()
        cases.append((kind, settings, s, cam, work, lens, focus))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        exes = list(pool.map(lambda c: _build_frame_harness(c[2], c[4]), cases))
    failed = []
    for (kind, settings, s, cam, work, lens, focus), exe in zip(cases, exes):
        hdr, fg = _run_frame_harness(exe, s, cam, work, lens, focus)
        if lens < 0:
            _, ref = oracle_py.render(s.desc(), cam, threads=2, want_hdr=True)
            pairs = [(hdr[j, :, :, :3], ref) for j in range(2)]
        else:
            r = oracle_py.render_film(s.desc(), cam, lens, focus, threads=2)
            pairs = [p for j in range(2) for p in ((hdr[j, :, :, :3], r["beauty"]), (hdr[j, :, :, 3], r["alpha"]),
                                                   (fg[j, :, :, :3], r["foreground"]))]
        bad = [int((np.ascontiguousarray(g).view(np.uint32) != w_.view(np.uint32)).sum()) for g, w_ in pairs]
        if any(bad):
            failed.append((kind, settings, lens, focus, bad))
    assert not failed, failed


BATCH_MAIN = r"""
#include "host_io.h"
#include "host_passes.h"
using namespace mm3e;
using namespace mm3e::wave;
// One wave of the batched form (mm3e_render_batch): a device-style job table of scenes with
// their own tapes, cameras and sizes, laid out as the batch engine lays it out (each job's
// samples, pixel slots and pixels after the previous job's), run as one pass sequence through
// the tape interpreter, then the resolve of every job's pixel slots.
int main(int argc, char** argv) {
    const uint32_t wlog = 3, nj = (uint32_t)std::atoi(argv[2]);
    std::vector<std::vector<float4>> tapes(nj);
    std::vector<FrameJob> jobs(nj);
    JobTotals tot{nj, 0, 0, 0};
    uint32_t levels = 1, lights = 0;
    bool ao = false, shadows = false;
    for (uint32_t k = 0; k < nj; ++k) {
        tapes[k] = read_words(argv[3 + 4 * k]);
        const unsigned char* tape = reinterpret_cast<const unsigned char*>(tapes[k].data());
        const TapeHeader& H = *tape_view(tape).h;
        FrameJob& J = jobs[k];
        J = FrameJob{};
        J.tape = tape;
        J.cam = read_camera(argv[4 + 4 * k]);
        J.width = (uint32_t)std::atoi(argv[5 + 4 * k]);
        J.height = (uint32_t)std::atoi(argv[6 + 4 * k]);
        J.aa = H.aa;
        J.spp = H.aa * H.aa;
        J.tiles_x = (J.width + 7u) / 8u;
        J.n_slots = J.tiles_x * ((J.height + 3u) / 4u) * 32u;
        J.n_samples = J.n_slots * J.spp;
        J.n_pixels = J.width * J.height;
        J.n_lights = H.n_lights;
        J.sample_base = tot.n_samples;
        J.slot_base = tot.n_slots;
        J.pixel_base = tot.n_pixels;
        tot.n_samples += J.n_samples;
        tot.n_slots += J.n_slots;
        tot.n_pixels += J.n_pixels;
        levels = levels > H.bounces + 1u ? levels : H.bounces + 1u;
        lights = lights > H.n_lights ? lights : H.n_lights;
        ao = ao || ((H.flags & SF_AO) && H.ao_samples > 0);
        shadows = shadows || ((H.flags & SF_SHADOWS) && H.shadow_steps > 0 && H.n_lights > 0);
    }
    HostFrame F;
    F.init(tot.n_samples, levels, lights, tot.n_pixels);
    WaveArgs a{};
    a.job0 = jobs[0];
    a.jobs = jobs.data();
    a.totals = &tot;
    a.n_jobs = nj;
    a.tile_wlog = wlog;
    host_levels_with<InterpField>(a, jobs[0].tape, SRC_SAMPLES, tot.n_samples, F, ao, shadows);
    for (uint32_t s = 0; s < tot.n_slots; ++s) resolve_slot(a, s, nj);
    FILE* fo = std::fopen(argv[1], "wb");
    std::fwrite(F.hdr.data(), sizeof(float4), F.hdr.size(), fo);
    std::fclose(fo);
    return 0;
}
"""


def test_batched_wave_equals_oracle_on_host(tmp_path):
    """A batched wave (the job-table path of march_kernels.cuh and shade_kernels.cuh: the job of a
    sample by binary search over the table, each lane's own job's tape, AO for AO jobs only, the
    per-job resolve) over scenes of different kinds, sizes, AA, bounce and light counts, with and
    without AO and shadows, compiled for the host and run as one pass sequence through the tape
    interpreter: every job's HDR pixels equal the oracle's render of its scene bit for bit."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    jobs = [scenes.gallery_scene(40, 24), scenes.spheres_scene(33, 17), scenes.hero_scene(24, 20, 2, 2),
            scenes.procedural_scene(3, 16, 9), _no_ao_samples_scene(), csg_zoo_scene(2, 20, 12),
            scenes.procedural_scene(8, 1, 1), scenes.cornell_scene(20, 20)]
    no_shadow, _ = jobs[1]
    no_shadow.shadows = False
    no_ao, _ = jobs[3]
    no_ao.ao = False
    (tmp_path / "main.cpp").write_text('#include "shade_kernels.cuh"\n' + BATCH_MAIN)
    exe = tmp_path / "batch"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS, str(tmp_path / "main.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    args = [str(exe), str(tmp_path / "out.bin"), str(len(jobs))]
    for k, (s, cam) in enumerate(jobs):
        (tmp_path / f"tape{k}.bin").write_bytes(mm3e_cuda.scene_tape(s))
        _cam_bin(cam, tmp_path / f"cam{k}.bin")
        d = s.desc().desc
        args += [str(tmp_path / f"tape{k}.bin"), str(tmp_path / f"cam{k}.bin"), str(d.width), str(d.height)]
    subprocess.run(args, check=True)
    hdr = np.fromfile(tmp_path / "out.bin", np.float32).reshape(-1, 4)
    base = 0
    for k, (s, cam) in enumerate(jobs):
        d = s.desc().desc
        n = d.width * d.height
        got = np.ascontiguousarray(hdr[base:base + n, :3]).reshape(d.height, d.width, 3)
        _, ref = oracle_py.render(s.desc(), cam, threads=2, want_hdr=True)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), \
            (k, int((got.view(np.uint32) != ref.view(np.uint32)).any(axis=2).sum()), n)
        base += n
    assert base == len(hdr)


POST_MAIN = r"""
#include "host_io.h"
#include "lower.h"
#include "march_kernels.cuh"  // its dynamic shared memory is extern: before __shared__ turns static
#undef __shared__
#define __shared__ static
#include "post_kernels.cuh"
using namespace mm3e;
using namespace mm3e::wave;
// The post of one frame as launch_post runs it, on a given HDR image: without bloom the resolve
// kernel; with bloom the fused bright-pass + horizontal blur (blocks of POST_THREADS threads
// sharing a window) and the vertical blur + resolve. Arguments: hdr, out, w, h, exposure, bloom,
// threshold, intensity, radius, format (0 RGBA8, 1 RGBA f32).
int main(int argc, char** argv) {
    const std::vector<float> hdr3 = read_floats(argv[1]);
    const uint32_t w = (uint32_t)std::atoi(argv[3]), h = (uint32_t)std::atoi(argv[4]), n = w * h;
    const float exposure = std::strtof(argv[5], nullptr), threshold = std::strtof(argv[7], nullptr);
    const float intensity = std::strtof(argv[8], nullptr);
    const bool bloom = std::atoi(argv[6]) != 0 && intensity > 0.0f;
    const uint32_t radius = (uint32_t)std::atoi(argv[9]), format = std::atoi(argv[10]) ? MM3E_FB_RGBA_F32 : MM3E_FB_RGBA8;
    const std::vector<float> weights = gaussian_kernel(bloom ? radius : 1u);  // as upload_post_kernel
    std::vector<float4> hdr(n), blur(n), out32(n);
    std::vector<uchar4> out8(n);
    for (uint32_t i = 0; i < n; ++i) hdr[i] = make_float4(hdr3[3 * i], hdr3[3 * i + 1], hdr3[3 * i + 2], 1.0f);
    FrameJob J{};
    J.width = w;
    J.height = h;
    J.n_pixels = n;
    J.bloom_w = weights.data();
    J.bloom_radius = (uint32_t)(weights.size() / 2);
    J.flags = bloom ? JF_BLOOM : 0u;
    J.threshold = threshold;
    J.intensity = intensity;
    J.exposure = exposure;
    J.format = format;
    J.out = format == MM3E_FB_RGBA8 ? (void*)out8.data() : (void*)out32.data();
    PostArgs p{};
    p.job0 = J;
    p.n_jobs = 1;
    p.n_pixels = n;
    p.any_bloom = bloom ? 1 : 0;
    p.hdr = hdr.data();
    p.blur_h = blur.data();
    const unsigned T = POST_THREADS;
    if (!bloom) {
        host_launch((n + T - 1) / T, T, [&] { k_resolve_post(p); });
    } else {
        host_launch((n + BLOOM_SEG - 1) / BLOOM_SEG, T, [&] { k_bloom_h(p); });
        const uint32_t groups = w * ((h + 3u) / 4u);
        host_launch((groups + T - 1) / T, T, [&] { k_bloom_v<true>(p); });
    }
    FILE* fo = std::fopen(argv[2], "wb");
    if (format == MM3E_FB_RGBA8) std::fwrite(out8.data(), sizeof(uchar4), n, fo);
    else std::fwrite(out32.data(), sizeof(float4), n, fo);
    std::fclose(fo);
    return 0;
}
"""

POST_CASES = [  # w, h, bloom radius, threshold, intensity, exposure, format (0 RGBA8, 1 RGBA f32)
    (64, 36, 12, 0.8, 0.6, 1.0, 0), (64, 36, 12, 0.8, 0.6, 1.0, 1), (1, 1, 12, 0.5, 0.6, 1.0, 0),
    (1, 9, 12, 0.5, 0.6, 1.3, 0), (9, 1, 3, 0.5, 0.6, 0.7, 0), (13, 7, 40, 0.2, 1.5, 1.0, 0),
    (37, 21, 0, 0.5, 0.6, 1.0, 0), (70, 3, 1, 0.0, 0.3, 2.0, 1), (33, 17, 12, 0.8, 0.0, 1.0, 0),
    (300, 5, 32, 0.6, 0.8, 1.0, 0), (300, 5, 33, 0.6, 0.8, 1.0, 0)]


def test_post_equals_oracle_on_host(tmp_path):
    """The post kernels (post_kernels.cuh: the fused bright-pass + horizontal blur with its
    swizzled shared window and four-output blur4, the vertical blur + resolve, the resolve
    without bloom; exposure, ACES, gamma and the RGBA8 or RGBA f32 write; post.rs:36-115),
    compiled for the host and run as blocks of POST_THREADS threads, on the oracle's own HDR image,
    against the oracle's post of that image: every byte (RGBA8) or bit (f32) equal. The cases
    cover 1x1, single rows and columns, radius 0, 1, 12, 32 and 33 (the latter two on either
    side of the shared window's halo) and 40, a threshold of 0 and bloom with intensity 0."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    flags = ["-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE, "-I", CSRC, "-I",
             HOST_DIR]
    r = subprocess.run(["g++"] + flags + ["-c", os.path.join(CSRC, "lower.cpp"), "-o", str(tmp_path / "lower.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    (tmp_path / "main.cpp").write_text(POST_MAIN)
    exe = tmp_path / "post"
    r = subprocess.run(["g++"] + flags + ["-include", SHIM, "-include", STUBS, str(tmp_path / "main.cpp"),
                                          str(tmp_path / "lower.o"), "-pthread", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    failed = []
    for k, (w, h, radius, thr, inten, exposure, fmt) in enumerate(POST_CASES):
        scene, cam = scenes.gallery_scene(w, h)
        scene.post.bloom = True
        scene.post.bloom_radius = radius
        scene.post.bloom_threshold = thr
        scene.post.bloom_intensity = inten
        scene.post.exposure = exposure
        handle = scene.desc()
        _, hdr = oracle_py.render(handle, cam, threads=2, want_hdr=True)
        ref = oracle_py.post(handle, hdr)
        hdr.astype(np.float32).tofile(tmp_path / f"hdr{k}.bin")
        post = scene.post
        subprocess.run([str(exe), str(tmp_path / f"hdr{k}.bin"), str(tmp_path / f"out{k}.bin"), str(w), str(h),
                        repr(float(post.exposure)), "1", repr(float(post.bloom_threshold)),
                        repr(float(post.bloom_intensity)), str(radius), str(fmt)], check=True)
        if fmt == 0:
            got = np.fromfile(tmp_path / f"out{k}.bin", np.uint8).reshape(h, w, 4)
            bad = int((got != mm3e_cuda.to_rgba8(ref)).any(-1).sum())
        else:
            got = np.fromfile(tmp_path / f"out{k}.bin", np.float32).reshape(h, w, 4)
            bad = int((got.view(np.uint32) != ref.view(np.uint32)).any(-1).sum())
        if bad:
            failed.append(((w, h, radius, thr, inten, exposure, fmt), bad))
    assert not failed, failed


def test_degenerate_cameras_equal_oracle_on_host(frame_harnesses, tmp_path):
    """Cameras the C ABI takes without checks, as the reference's render does: a NaN or infinite
    eye, an eye 1e7 away, zero basis vectors, and a zero, negative, NaN or huge field-of-view
    scale. Whole frames through the device pass sequence equal the oracle's render bit for bit
    (NaN for NaN) over both fields; every march ends within its step budget."""
    from mm3e_cuda.abi import Camera
    scene, cam = FRAME_SCENES["gallery"]()
    exe = frame_harnesses[mm3e_cuda.spec_source(scene)]
    nan, inf = float("nan"), float("inf")

    def variant(eye=None, fwd=None, right=None, up=None, fov=None):
        c = Camera()
        c.eye[:] = eye or list(cam.eye)
        c.forward[:] = fwd or list(cam.forward)
        c.right[:] = right or list(cam.right)
        c.up[:] = up or list(cam.up)
        c.fov_scale = cam.fov_scale if fov is None else fov
        return c

    cases = {"nan_eye": variant(eye=[nan, 1.0, 1.0]), "inf_eye": variant(eye=[inf, 1.0, -5.0]),
             "far_eye": variant(eye=[1e7, 2.0, -1e7]), "zero_forward": variant(fwd=[0.0, 0.0, 0.0]),
             "zero_basis": variant(fwd=[0.0, 0.0, 0.0], right=[0.0, 0.0, 0.0], up=[0.0, 0.0, 0.0]),
             "fov_zero": variant(fov=0.0), "fov_negative": variant(fov=-1.0), "fov_nan": variant(fov=nan),
             "fov_huge": variant(fov=1e30)}
    failed = {}
    for name, c in cases.items():
        out, _ = _run_frame_harness(exe, scene, c, tmp_path)
        _, ref = oracle_py.render(scene.desc(), c, threads=2, want_hdr=True)
        for k in range(2):
            dev = np.ascontiguousarray(out[k, :, :, :3])
            same = (dev.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(dev) & np.isnan(ref))
            if not same.all():
                failed[(name, k)] = int((~same).any(axis=2).sum())
    assert not failed, failed


DEGENERATE_OBJECTS = {  # one extra object in the spheres scene
    "tiny_sphere": (lambda: Prim.sphere(1e-30), Transform((0.5, 0.5, -1.0))),
    "huge_sphere": (lambda: Prim.sphere(1e20), Transform((0.0, -1e20 - 5.0, 0.0))),
    "far_object": (lambda: Prim.sphere(1.0), Transform((1e18, 0.0, 0.0))),
    "tiny_scale": (lambda: Prim.box((1.0, 1.0, 1.0)), Transform((0.0, 0.5, -2.0), scale=1e-20)),
    "huge_scale": (lambda: Prim.torus(1.0, 0.2), Transform((0.0, 0.5, 50.0), scale=1e15)),
    "zero_box": (lambda: Prim.box((0.0, 0.0, 0.0)), Transform((0.3, 0.5, -1.0))),
    "fat_torus": (lambda: Prim.torus(0.2, 1.0), Transform((0.0, 1.0, -1.5))),
    "zero_capsule": (lambda: Prim.capsule((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.0), Transform((0.0, 1.0, -1.0))),
    "flat_ellipsoid": (lambda: Prim.ellipsoid((1.0, 0.0, 1.0)), Transform((0.0, 1.5, -1.0))),
    "negative_radius": (lambda: Prim.sphere(-0.5), Transform((0.0, 1.0, -1.0))),
}


def test_degenerate_objects_equal_oracle_on_host(tmp_path):
    """Objects at the edges of their parameters, which the reference's validation accepts: radii
    of 1e-30, 1e20 and -0.5, a sphere 1e18 away, scales of 1e-20 and 1e15, a zero box and a zero
    capsule, a torus fatter than its ring, a flat ellipsoid. Whole frames through the device pass
    sequence equal the oracle's render bit for bit over both fields: the generated field's culls
    and weak bounds stay exact there too."""
    from concurrent.futures import ThreadPoolExecutor
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    cases = []
    for name, (prim, tr) in DEGENERATE_OBJECTS.items():
        s, cam = scenes.spheres_scene(24, 14)
        s.add(Object(prim(), tr, len(cases) % 3 + 1))
        assert mm3e_cuda.validate(s)[0] == abi.OK, name
        work = tmp_path / name
        work.mkdir()
        cases.append((name, s, cam, work))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        exes = list(pool.map(lambda c: _build_frame_harness(c[1], c[3]), cases))
    failed = {}
    for (name, s, cam, work), exe in zip(cases, exes):
        out, _ = _run_frame_harness(exe, s, cam, work)
        _, ref = oracle_py.render(s.desc(), cam, threads=2, want_hdr=True)
        for k in range(2):
            dev = np.ascontiguousarray(out[k, :, :, :3])
            same = (dev.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(dev) & np.isnan(ref))
            if not same.all():
                failed[(name, k)] = int((~same).any(axis=2).sum())
    assert not failed, failed
