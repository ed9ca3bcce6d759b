"""The other device paths, compiled for the host (host_checks.py): the GI bake, the preview path
(G-buffer, reprojection, hybrid), a batched wave of jobs and the post kernels, against the
oracle's results bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from mm3e_cuda import scenes
from mm3e_cuda.scene import orbit_camera, radians
from field_scenes import csg_zoo_scene
from host_checks import (CSRC, CUDA_INCLUDE, HOST_DIR, SCENES, SHIM, STUBS, cam_bin, harness_source, no_ao_samples_scene,
                         spec_namespace)

GI_MAIN = harness_source("gi_bake.inc")


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
    defines, ns = spec_namespace(scene)
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


PREVIEW_MAIN = harness_source("preview.inc")


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
    defines, ns = spec_namespace(scene)
    (tmp_path / "main.cpp").write_text(defines + '#include "shade_kernels.cuh"\n#include "reproject_kernels.cuh"\n'
                                       'namespace mm3e { namespace spec {\n' + ns + "\n}}\n" + PREVIEW_MAIN)
    exe = tmp_path / "preview"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE,
                        "-I", CSRC, "-I", HOST_DIR, "-include", SHIM, "-include", STUBS, str(tmp_path / "main.cpp"),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    (tmp_path / "tape.bin").write_bytes(mm3e_cuda.scene_tape(scene))
    cam_bin(c0, tmp_path / "c0.bin")
    cam_bin(c1, tmp_path / "c1.bin")
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


BATCH_MAIN = harness_source("batch_wave.inc")


def test_batched_wave_equals_oracle_on_host(tmp_path):
    """A batched wave (the job-table path of march_kernels.cuh and shade_kernels.cuh: the job of a
    sample by binary search over the table, each lane's own job's tape, AO for AO jobs only, the
    per-job resolve) over scenes of different kinds, sizes, AA, bounce and light counts, with and
    without AO and shadows, compiled for the host and run as one pass sequence through the tape
    interpreter: every job's HDR pixels equal the oracle's render of its scene bit for bit. The
    multi-job post that follows (post_kernels.cuh with the job table: each pixel's job by binary
    search, each job's own bloom kernel, threshold, intensity and exposure, bloom off for some)
    gives every job's RGBA8 bytes of the oracle's frame."""
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    jobs = [scenes.gallery_scene(40, 24), scenes.spheres_scene(33, 17), scenes.hero_scene(24, 20, 2, 2),
            scenes.procedural_scene(3, 16, 9), no_ao_samples_scene(), csg_zoo_scene(2, 20, 12),
            scenes.procedural_scene(8, 1, 1), scenes.cornell_scene(20, 20)]
    no_shadow, _ = jobs[1]
    no_shadow.shadows = False
    no_ao, _ = jobs[3]
    no_ao.ao = False
    jobs[1][0].post.bloom_radius = 3
    jobs[2][0].post.bloom = False
    jobs[5][0].post.bloom_threshold, jobs[5][0].post.bloom_intensity, jobs[5][0].post.bloom_radius = 0.2, 0.8, 33
    jobs[7][0].post.exposure = 1.5
    (tmp_path / "main.cpp").write_text('#include "shade_kernels.cuh"\n' + BATCH_MAIN)
    exe = tmp_path / "batch"
    flags = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", CUDA_INCLUDE, "-I", CSRC, "-I",
             HOST_DIR]
    r = subprocess.run(flags + ["-c", os.path.join(CSRC, "lower.cpp"), "-o", str(tmp_path / "lower.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run(flags + ["-include", SHIM, "-include", STUBS, str(tmp_path / "main.cpp"), str(tmp_path / "lower.o"),
                                "-pthread", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    args = [str(exe), str(tmp_path / "out.bin"), str(len(jobs))]
    for k, (s, cam) in enumerate(jobs):
        (tmp_path / f"tape{k}.bin").write_bytes(mm3e_cuda.scene_tape(s))
        cam_bin(cam, tmp_path / f"cam{k}.bin")
        d = s.desc().desc
        args += [str(tmp_path / f"tape{k}.bin"), str(tmp_path / f"cam{k}.bin"), str(d.width), str(d.height)]
    subprocess.run(args, check=True)
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    total = sum(s.desc().desc.width * s.desc().desc.height for s, _ in jobs)
    hdr = raw[:total * 16].view(np.float32).reshape(-1, 4)
    rgba8 = raw[total * 16:]
    assert len(rgba8) == total * 4
    base = 0
    for k, (s, cam) in enumerate(jobs):
        d = s.desc().desc
        n = d.width * d.height
        got = np.ascontiguousarray(hdr[base:base + n, :3]).reshape(d.height, d.width, 3)
        rgba, ref = oracle_py.render(s.desc(), cam, threads=2, want_hdr=True)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), \
            (k, int((got.view(np.uint32) != ref.view(np.uint32)).any(axis=2).sum()), n)
        got8 = rgba8[base * 4:(base + n) * 4].reshape(d.height, d.width, 4)
        want8 = mm3e_cuda.to_rgba8(rgba)
        assert np.array_equal(got8, want8), (k, "rgba8", int((got8 != want8).any(-1).sum()), n)
        base += n
    assert base == total


POST_MAIN = harness_source("post.inc")


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
