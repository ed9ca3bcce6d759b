"""Shared pieces of the host-compiled device-code checks (test_host_field_cpu.py,
test_host_frame_cpu.py, test_host_paths_cpu.py).

The device code (device_math.cuh, march_kernels.cuh, shade_kernels.cuh, post_kernels.cuh,
reproject_kernels.cuh and a scene's generated field) compiles as plain C++ with the host
definitions in tests/host_field: exact intrinsics (host_shim.h), warp builtins and block
emulation (host_kernel_stubs.h), file readers (host_io.h) and the pass sequence (host_passes.h).
The harnesses in tests/host_field/*.inc drive it item by item, and the tests compare the results
with the oracle's bit for bit. On the host both sides call the same libm, so the device code's
operation order is pinned without a GPU; on the device only CUDA's transcendental functions
differ. This module holds the paths, the seeded scenes and the frame harness's build and run."""
import os
import subprocess
from math import radians

import numpy as np

import mm3e_cuda
import oracle_py
from mm3e_cuda import scenes
from mm3e_cuda.scene import Material, Object, Prim, Scene, SdfVolume, GiVolume, Transform, directional, look_at, orbit_camera
from field_scenes import csg_zoo_scene, noncons_scene, planes_scene, smooth_chain_scene, unbounded_mix_scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


CSRC = os.path.join(ROOT, "atom-3d-engine_gb300", "csrc")


HOST_DIR = os.path.join(ROOT, "tests", "host_field")


SHIM = os.path.join(HOST_DIR, "host_shim.h")


CUDA_INCLUDE = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def harness_source(name):
    """Source of a host harness in tests/host_field."""
    with open(os.path.join(HOST_DIR, name)) as f:
        return f.read()


STUBS = os.path.join(HOST_DIR, "host_kernel_stubs.h")


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


FRAME_MAIN = harness_source("frame.inc")


def cornell_gi_scene():
    """The Cornell room with a GI probe volume baked by the oracle (6x6x6 probes, 4 samples)."""
    scene, cam = scenes.cornell_scene(64, 36)
    mn, size, dims, cubes = oracle_py.bake_gi(scene.desc(), (6, 6, 6), 4)
    scene.gi = GiVolume(mn, size, dims, cubes)
    return scene, cam


def volume_scene():
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


def no_ao_samples_scene():
    """The gallery with AO on but no AO samples: ambient_occlusion then returns 1 (march.rs:266)."""
    s, cam = scenes.gallery_scene(64, 36)
    s.marcher.ao_samples = 0
    return s, cam


def shading_zoo_scene():
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


FRAME_SCENES = {**SCENES, "cornell_gi": cornell_gi_scene, "volumes": volume_scene,
                "no_ao_samples": no_ao_samples_scene, "shading_zoo": shading_zoo_scene}


def build_frame_harness(scene, work):
    """Compile the frame harness with the scene's generated field into `work`; its path."""
    defines, ns = spec_namespace(scene)
    (work / "main.cpp").write_text(defines + '#include "shade_kernels.cuh"\nnamespace mm3e { namespace spec {\n' + ns +
                                   "\n}}\n" + FRAME_MAIN)
    exe = work / "frame"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS, str(work / "main.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def run_frame_harness(exe, scene, cam, work, lens=-1.0, focus=1.0):
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


def cam_bin(cam, path):
    np.array(list(cam.eye) + list(cam.forward) + list(cam.right) + list(cam.up) + [cam.fov_scale],
             np.float32).tofile(path)


def random_case(rng):
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


def spec_namespace(scene):
    """The scene's generated field for a host harness: (defines, body of `namespace spec`)."""
    src = mm3e_cuda.spec_source(scene)
    ns = src[src.index("namespace spec {") + len("namespace spec {"):src.index("}  // namespace spec")]
    defines = "#define MM3E_SHARED_SINCOS 1\n" if "#define MM3E_SHARED_SINCOS 1" in src else ""
    return defines, ns


GXX = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w"]


def compile_harnesses(jobs, exe_name):
    """Compile each job's main.cpp in parallel. jobs: name -> (directory, extra g++ flags);
    returns name -> executable path."""
    from concurrent.futures import ThreadPoolExecutor

    def one(job):
        d, flags = job
        exe = d / exe_name
        r = subprocess.run(GXX + ["-I", CUDA_INCLUDE, "-I", CSRC, "-I", HOST_DIR] + flags + [str(d / "main.cpp"), "-o", str(exe)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        return exe

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        exes = list(pool.map(one, jobs.values()))
    return dict(zip(jobs, exes))
