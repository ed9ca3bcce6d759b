"""Whole frames through the device pass sequence, compiled for the host (host_checks.py): HDR
frames, film frames, AOV modes, frames at the edges of the scene's and marcher's settings, seeded
random configurations and degenerate inputs, each over both the tape interpreter's field and the
scene's generated field, against the oracle's render bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from mm3e_cuda import abi, scenes
from mm3e_cuda.scene import Object, Prim, Transform
from host_checks import (CSRC, CUDA_INCLUDE, FRAME_SCENES, HOST_DIR, SHIM, STUBS, build_frame_harness, harness_source,
                         random_case, run_frame_harness)

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
        exes = list(pool.map(build_frame_harness, by_src.values(), works))
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
    out, _ = run_frame_harness(frame_harnesses[mm3e_cuda.spec_source(scene)], scene, cam, tmp_path)
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
    hdr, fg = run_frame_harness(frame_harnesses[mm3e_cuda.spec_source(scene)], scene, cam, tmp_path, lens, focus)
    ref = oracle_py.render_film(scene.desc(), cam, lens, focus, threads=2)
    assert 0.0 < ref["alpha"].mean() < 1.0 and ref["beauty"].std() > 0.1
    for k, label in enumerate(("interpreter", "specialised")):
        for got, want, what in ((hdr[k, :, :, :3], ref["beauty"], "beauty"), (hdr[k, :, :, 3], ref["alpha"], "alpha"),
                                (fg[k, :, :, :3], ref["foreground"], "foreground")):
            got = np.ascontiguousarray(got)
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
                (label, what, int((got.view(np.uint32) != want.view(np.uint32)).sum()))


AOV_MAIN = harness_source("aov.inc")


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
        exes = dict(zip(cases, pool.map(lambda c: build_frame_harness(c[0], c[2]), cases.values())))
    failed = {}
    for edge, (scene, cam, work) in cases.items():
        out, _ = run_frame_harness(exes[edge], scene, cam, work)
        _, ref = oracle_py.render(scene.desc(), cam, threads=2, want_hdr=True)
        for k, label in enumerate(("interpreter", "specialised")):
            dev = np.ascontiguousarray(out[k, :, :, :3])
            bad = int((dev.view(np.uint32) != ref.view(np.uint32)).any(axis=2).sum())
            if bad:
                failed[(edge, label)] = bad
    assert not failed, failed


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
        kind, settings, s, cam = random_case(rng)
        lens, focus = (rng.choice([0.02, 0.1, 0.4]), rng.choice([0.5, 3.0, 7.0, 20.0])) if k % 2 else (-1.0, 1.0)
        work = tmp_path / str(k)
        work.mkdir()
        cases.append((kind, settings, s, cam, work, lens, focus))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as pool:
        exes = list(pool.map(lambda c: build_frame_harness(c[2], c[4]), cases))
    failed = []
    for (kind, settings, s, cam, work, lens, focus), exe in zip(cases, exes):
        hdr, fg = run_frame_harness(exe, s, cam, work, lens, focus)
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
        out, _ = run_frame_harness(exe, scene, c, tmp_path)
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
        exes = list(pool.map(lambda c: build_frame_harness(c[1], c[3]), cases))
    failed = {}
    for (name, s, cam, work), exe in zip(cases, exes):
        out, _ = run_frame_harness(exe, s, cam, work)
        _, ref = oracle_py.render(s.desc(), cam, threads=2, want_hdr=True)
        for k in range(2):
            dev = np.ascontiguousarray(out[k, :, :, :3])
            same = (dev.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(dev) & np.isnan(ref))
            if not same.all():
                failed[(name, k)] = int((~same).any(axis=2).sum())
    assert not failed, failed
