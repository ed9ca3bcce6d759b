#!/usr/bin/env python
"""Benchmark of the GB300 per-pixel SDF render path (one JSON line on rank 0).

Workload (default): the 1080p feature gallery (1920x1080, aa 1, one reflection bounce, soft
shadows, AO, fog, sky IBL, bloom + ACES; 11 primitives, smooth union, twist/bend/onion/round/
repeat/mirror; max 256 steps). A step = `--frames-per-step` frames (32 by default) of the same
scene and camera, each rendered on the GPU from the resident scene tape to a device RGBA8
framebuffer (render kernels + post kernels); the L2 is flushed between timed steps.

  value      frames/s with the scene resident in HBM (CUDA events on the render stream)
  e2e        frames/s through the public C ABI call mm3e_render with a host framebuffer:
             per frame the camera goes host->device and the RGBA8 frame device->host (on a
             host whose page tables the GPU shares, the post kernel stores it straight into
             the caller's buffer over NVLink-C2C; elsewhere through a pinned staging copy)
  roofline   FP32-pipe roofline of the dominant kernel: the algorithmic f32 operations of its
             phase per frame (oracle operation count split by kernel, committed fixture) / its
             CUDA-event-timed device time per frame (events around every pass, a second run of
             the same frames), against SMs x 128 lanes x 2 x max SM clock
  cpu_baseline  the CPU restatement of the reference render path on all host cores, whole frames
  parity     the last timed frame against the oracle's frame of the cpu_baseline leg, and the
             primary hits against the oracle's

--impl reference times the CPU reference path (the oracle restatement: the Rust reference has no
toolchain here) on the same workload, one whole frame per step, and prints its own line with the
same `config`; it builds its scene through the oracle's helpers and never loads the CUDA library.
Multi-GPU runs are replicas: each rank renders its own frames (scaling "weak").
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "atom-3d-engine_gb300"))

COUNTS_FIXTURE = os.path.join(ROOT, "tests", "golden", "workload_counts.json")

# DRAM bytes (read + write) of one primary-level march launch (the scene-specialised kernel in the
# timed launch shape), from an ncu capture of the same kernel on the workload at 960x540
# (71,168 + 0 bytes), scaled by the pixel ratio to the bench resolution: the tape lives in shared
# memory and the queues in L2, so DRAM traffic is small.
MARCH_DRAM_BYTES_960x540 = {"gallery_1080p": 70912}


def workloads(size=None):
    """Workload name -> () -> (Scene, Camera). `size` (w, h) overrides the resolution (small
    cases for profiler captures)."""
    from mm3e_cuda import scenes

    def sz(w, h):
        return size if size else (w, h)

    return {
        "gallery_1080p": lambda: scenes.gallery_scene(*sz(1920, 1080)),
        "spheres_540p": lambda: scenes.spheres_scene(*sz(960, 540)),
        "hero_540p_aa2": lambda: scenes.hero_scene(*sz(960, 540), 2, 2),
    }


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--frames-per-step", type=int, default=32,
                    help="frames of the workload (same scene and camera) rendered per timed step")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gallery_1080p")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline sample time")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="only render this many frames of the workload (no timing, no JSON line): the "
                         "command profilers run")
    ap.add_argument("--size", default=None, help="WxH resolution override (with --profile-frames)")
    ap.add_argument("--batch-scenes", type=int, default=256, help="scenes of the batched-form measurement")
    ap.add_argument("--served-seconds", type=float, default=2.0,
                    help="arrival window per rate of the served-form measurement (the full spec is 60)")
    ap.add_argument("--served-rates", default="200,1000,5000",
                    help="Poisson arrival rates (requests/s) of the served-form measurement")
    ap.add_argument("--served-only", action="store_true",
                    help="run only the served-form measurement and print it as its own JSON line")
    ap.add_argument("--served-max-requests", type=int, default=2000,
                    help="cap on requests per rate (the arrival window shrinks to fit)")
    ap.add_argument("--no-forms", action="store_true", help="skip the Cornell / batched / served measurements")
    ap.add_argument("--no-spec", action="store_true", help="time the tape interpreter (no NVRTC specialisation)")
    ap.add_argument("--tuning", default=None,
                    help="block,tile_wlog,unroll,min_blocks launch shape for the workload scene instead of the search")
    return ap.parse_args()


def _pct(v, q):
    import numpy as np

    return float(np.percentile(np.asarray(v, np.float64), q)) if len(v) else None


def bench_cornell(ctx, stream, torch):
    """Cornell GI room at 1920x1080: GPU probe bake (32^3 ambient cubes, 5 rays per face) from the
    tape, then frames through the plain call (L2 flushed between frames)."""
    from mm3e_cuda import abi, scenes

    import mm3e_cuda

    s, cam = scenes.cornell_scene(1920, 1080)
    cs = mm3e_cuda.CompiledScene(ctx, s)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    cs.bake_gi((32, 32, 32), 5)  # warm-up (first-use allocations)
    t0 = time.perf_counter()
    cs.bake_gi((32, 32, 32), 5)
    bake_s = time.perf_counter() - t0
    cs.specialize(cs.SPEC_AUTO)  # after the bake (a bake re-lowers the scene)
    out = torch.empty(1920 * 1080 * 4, dtype=torch.uint8, device="cuda")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    for _ in range(3):
        cs.render_device(cam, abi.FB_RGBA8, out.data_ptr(), out.numel())
    ms = []
    with torch.cuda.stream(stream):
        for i in range(10):
            flush.fill_(float(i))
            ev[0].record(stream)
            cs.render_device(cam, abi.FB_RGBA8, out.data_ptr(), out.numel())
            ev[1].record(stream)
            stream.synchronize()
            ms.append(ev[0].elapsed_time(ev[1]))
    specialized = cs.specialized
    cs.close()
    return {"workload": "cornell_gi_1080p", "frames_per_s": 1000.0 / statistics.median(ms),
            "frame_ms_median": statistics.median(ms), "gi_probes": "32^3 ambient cubes, 5 rays per face",
            "gi_bake_ms_host_wall": bake_s * 1000.0, "gi_bake_rays": 32 ** 3 * 6 * 5,
            "field": "scene-specialised (NVRTC)" if specialized else "tape interpreter"}


def bench_preview(ctx, torch, with_cpu):
    """Preview path at 1920x1080 on the gallery scene: render_gbuffer, then the camera moved 0.2
    along its right axis and the frame reprojected (row fill) and hybrid-reprojected (holes
    re-rendered). Host buffers in and out, host wall time per call (median of 5 after a warm-up).
    CPU leg: the oracle's G-buffer frame on all host cores and its hybrid reprojection."""
    import numpy as np

    from mm3e_cuda import scenes
    from mm3e_cuda.scene import look_at

    import mm3e_cuda

    s, c0 = scenes.gallery_scene(1920, 1080)
    eye, fwd, right = (np.array(c0.eye[:], np.float32), np.array(c0.forward[:], np.float32),
                       np.array(c0.right[:], np.float32))
    e1 = eye + np.float32(0.2) * right
    c1 = look_at(tuple(float(x) for x in e1), tuple(float(x) for x in e1 + fwd), (0.0, 1.0, 0.0),
                 2.0 * math.atan(c0.fov_scale))
    cs = mm3e_cuda.CompiledScene(ctx, s)
    cs.specialize(cs.SPEC_AUTO)

    def wall(fn, k=5):
        fn()
        ts = []
        for _ in range(k):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = fn()
            ts.append((time.perf_counter() - t0) * 1000.0)
        return statistics.median(ts), out

    g_ms, g = wall(lambda: cs.render_gbuffer(c0))
    r_ms, _ = wall(lambda: ctx.reproject(g, c1))
    h_ms, hyb = wall(lambda: ctx.reproject(g, c1, hybrid_scene=cs))
    full_ms, truth = wall(lambda: cs.render_gbuffer(c1))
    cs.close()
    out = {"workload": "gallery_1080p_preview", "camera_move": "0.2 along the camera's right axis",
           "render_gbuffer_ms": g_ms, "reproject_ms": r_ms, "reproject_hybrid_ms": h_ms,
           "hybrid_matches_full_view": float((hyb == truth["color"]).all(-1).mean()),
           "timing": "host wall per call, host buffers (H2D / D2H inside)"}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = oracle_py.render_gbuffer(s.desc(), c0, threads=threads)
        t_g = time.perf_counter() - t0
        t0 = time.perf_counter()
        oracle_py.reproject(ref, c0, c1, hybrid_handle=s.desc(), threads=threads)
        t_h = time.perf_counter() - t0
        out["cpu_baseline"] = {"render_gbuffer_ms": t_g * 1000.0, "reproject_hybrid_ms": t_h * 1000.0,
                               "cores": threads, "kind": "port", "sample": "one full 1920x1080 frame each"}
    return out


# The reference's published GPU numbers for its own benchmark scene (mm3e-gpu examples, RTX 5070 Ti
# over wgpu; README.md:15 and CHANGELOG.md:75-76), quoted beside ours on the same scene and loop.
PUBLISHED_GPU_RENDER_FPS = 698.9
PUBLISHED_RESOLUTION_FPS = {"960x540": 606.0, "1920x1080": 167.0, "2560x1440": 96.0, "3840x2160": 43.0}
SWEEP_SHAPES = [{"block": 128, "tile_wlog": t, "unroll": 64, "min_blocks": 0} for t in (2, 3, 5)]


def bench_published(ctx, stream, torch):
    """The reference's own GPU benchmarks re-run here: gpu_render.rs (960x540, aa 2, 3 bounces,
    120 frames of an orbiting camera, each rendered and read back as RGBA8: e2e through
    mm3e_render into one host framebuffer) and gpu_resolution.rs (the same scene at 540p to 4K,
    render only: device time per frame with CUDA events)."""
    import numpy as np

    from mm3e_cuda import abi, scenes

    import mm3e_cuda

    s, cam = scenes.gpu_render_scene(960, 540)
    cs = mm3e_cuda.CompiledScene(ctx, s)
    best, _ = cs.autotune(cam, spec_mode=cs.SPEC_AUTO)
    host = np.zeros((s.height, s.width, 4), np.uint8)
    cams = [scenes.gpu_render_scene(960, 540, 0.55 + i * 0.01)[1] for i in range(120)]
    for c in cams[:5]:
        cs.render(c, fmt=abi.FB_RGBA8, out=host)
    t0 = time.perf_counter()
    for c in cams:
        cs.render(c, fmt=abi.FB_RGBA8, out=host)
    loop_s = time.perf_counter() - t0
    cs.close()
    out = {"scene": "mm3e-gpu gpu_render.rs: hero scene, aa 2, 3 bounces, soft sun", "tuning": best,
           "gpu_render_960x540": {"frames_per_s": 120 / loop_s, "frames": 120,
                                  "timing": "host wall of the 120-frame orbit loop, render + RGBA8 readback per frame",
                                  "reference_published_fps": PUBLISHED_GPU_RENDER_FPS,
                                  "reference_hardware": "RTX 5070 Ti, wgpu (README.md:15)"}}
    sweep = {}
    for key in PUBLISHED_RESOLUTION_FPS:
        w, h = (int(v) for v in key.split("x"))
        s, cam = scenes.gpu_render_scene(w, h)
        cs = mm3e_cuda.CompiledScene(ctx, s)
        # per resolution: the 960x540 winner and the shapes that won at other sizes
        cands = [best] + [c for c in SWEEP_SHAPES if c != best]
        cs.autotune(cam, spec_mode=cs.SPEC_AUTO, candidates=cands, repeats=3)
        dev = torch.empty(w * h * 4, dtype=torch.uint8, device="cuda")
        for _ in range(3):
            cs.render_device(cam, abi.FB_RGBA8, dev.data_ptr(), dev.numel())
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
        with torch.cuda.stream(stream):
            for a, b in ev:
                a.record(stream)
                cs.render_device(cam, abi.FB_RGBA8, dev.data_ptr(), dev.numel())
                b.record(stream)
        stream.synchronize()
        ms = statistics.median(a.elapsed_time(b) for a, b in ev)
        sweep[key] = {"frames_per_s": 1000.0 / ms, "reference_published_fps": PUBLISHED_RESOLUTION_FPS[key]}
        cs.close()
    out["gpu_resolution_render_only"] = sweep
    out["gpu_resolution_note"] = "reference: RTX 5070 Ti, wgpu, render-only (CHANGELOG.md:75-76)"
    return out


def bench_batched(ctx, stream, torch, n_scenes):
    """Batched form: n seeded procedural scenes (8-64 primitives, random CSG, mixed resolutions
    256^2 / 512^2 / 1280x720 / 1920x1080, orbit cameras) rendered as one batch (autotuned launch
    shape, CUDA-graph pass sequences) vs the plain per-frame call of every scene in turn."""
    from mm3e_cuda import abi, scenes

    import mm3e_cuda

    items = [scenes.procedural_scene(seed) for seed in range(n_scenes)]
    compiled = [mm3e_cuda.CompiledScene(ctx, s) for s, _ in items]
    outs = [torch.empty(s.width * s.height * 4, dtype=torch.uint8, device="cuda") for s, _ in items]
    pixels = sum(s.width * s.height for s, _ in items)
    jobs = ctx.make_jobs([(c, cam, 0, 0, abi.FB_RGBA8, o.data_ptr(), None)
                          for c, (s, cam), o in zip(compiled, items, outs)])
    ctx.configure_batch(max_samples=1 << 28, use_graphs=True)  # all 256 scenes in one pass sequence
    t0 = time.perf_counter()
    best, table = ctx.autotune(ctx.make_jobs([(c, cam, 0, 0, abi.FB_RGBA8, o.data_ptr(), None)
                                              for c, (s, cam), o in list(zip(compiled, items, outs))[:32]]))
    tune_s = time.perf_counter() - t0
    ctx.render_batch(jobs)  # warm-up: graphs captured, buffers grown
    batch_ms, stats = [], None
    for _ in range(3):
        stats = ctx.render_batch(jobs)
        batch_ms.append(stats["device_ms"])
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for c, (s, cam), o in zip(compiled, items, outs):  # warm-up: per-scene buffers
        c.render_device(cam, abi.FB_RGBA8, o.data_ptr(), o.numel())
    ctx.sync()
    plain_ms = []
    with torch.cuda.stream(stream):
        for _ in range(2):
            ev[0].record(stream)
            for c, (s, cam), o in zip(compiled, items, outs):
                c.render_device(cam, abi.FB_RGBA8, o.data_ptr(), o.numel())
            ev[1].record(stream)
            stream.synchronize()
            plain_ms.append(ev[0].elapsed_time(ev[1]))
    b = statistics.median(batch_ms)
    p = statistics.median(plain_ms)
    # per resolution class: that class's frames as one batch against the plain call of each
    by_res = {}
    for res in sorted({(s.width, s.height) for s, _ in items}, key=lambda r: r[0] * r[1]):
        idx = [i for i, (s, _) in enumerate(items) if (s.width, s.height) == res]
        cjobs = ctx.make_jobs([(compiled[i], items[i][1], 0, 0, abi.FB_RGBA8, outs[i].data_ptr(), None) for i in idx])
        ctx.render_batch(cjobs)
        cb = statistics.median(ctx.render_batch(cjobs)["device_ms"] for _ in range(2))
        cp = []
        with torch.cuda.stream(stream):
            for _ in range(2):
                ev[0].record(stream)
                for i in idx:
                    compiled[i].render_device(items[i][1], abi.FB_RGBA8, outs[i].data_ptr(), outs[i].numel())
                ev[1].record(stream)
                stream.synchronize()
                cp.append(ev[0].elapsed_time(ev[1]))
        cpm = statistics.median(cp)
        by_res[f"{res[0]}x{res[1]}"] = {"frames": len(idx), "batch_ms": cb, "plain_ms": cpm,
                                        "batched_over_plain": cpm / cb}
    for c in compiled:
        c.close()
    return {"workload": f"procedural_batch_{n_scenes}", "frames": n_scenes, "pixels": pixels, "by_resolution": by_res,
            "batched_frames_per_s": n_scenes * 1000.0 / b, "batched_mrays_per_s_primary": pixels / b / 1e3,
            "plain_frames_per_s": n_scenes * 1000.0 / p, "batched_over_plain": p / b,
            "batch_ms": b, "plain_ms": p, "sequences": stats["sequences"],
            "kernel_launches": stats["kernel_launches"], "graph_launches": stats["graph_launches"],
            "tuning": best, "autotune_s": tune_s, "autotune_table": table}


def bench_served(ctx_factory, seconds, max_requests, rates=(200, 1000, 5000), seed=7, spec_workers=12):
    """Served form: Poisson arrivals at each rate; 70% camera updates of resident procedural
    scenes, 20% new procedural scenes, 10% scenes around a 128^3 grid baked on the GPU from a
    seeded displaced icosphere (subdivision 5); HBM budget 40 GB. The same trace replayed through
    the served form (continuous batching; the resident scenes' specialised kernels compiled on
    `spec_workers` host threads before the stream starts) and through the plain per-request
    launch (one at a time, the tape interpreter)."""
    import numpy as np

    import mm3e_cuda
    from mm3e_cuda import scenes
    from mm3e_cuda.scene import SdfVolume, orbit_camera

    rng = np.random.default_rng(seed)
    resident = [scenes.procedural_scene(1000 + i) for i in range(64)]
    fresh = [scenes.procedural_scene(5000 + i) for i in range(32)]
    meshes = [scenes.displaced_icosphere(k, 5) for k in range(4)]
    placeholder = SdfVolume((2, 2, 2), (0, 0, 0), (1, 1, 1), np.zeros(8, np.float32))
    mesh_scenes = []
    for k in range(4):
        s, cam = scenes.mesh_volume_scene(placeholder, seed=k, width=512, height=512)
        s.marcher.normal_h = 0.02
        mesh_scenes.append((s, cam))
    bufs = {}

    def out_for(w, h):
        lst = bufs.setdefault((w, h), [np.zeros((h, w, 4), np.uint8) for _ in range(4)])
        return lst[int(rng.integers(0, len(lst)))]

    results = {}
    for rate in rates:
        n = int(min(max_requests, rate * seconds))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
        kinds = rng.random(n)
        plan = []
        for i in range(n):
            if kinds[i] < 0.7:
                j = int(rng.integers(0, len(resident)))
                s, _ = resident[j]
                cam = orbit_camera((0.0, 0.0, 0.0), float(rng.uniform(9, 15)), float(rng.uniform(-3.1, 3.1)),
                                   float(rng.uniform(0.1, 0.7)), 0.8)
                plan.append(("resident", j, cam, s.width, s.height))
            elif kinds[i] < 0.9:
                j = int(rng.integers(0, len(fresh)))
                plan.append(("new", j, fresh[j][1], fresh[j][0].width, fresh[j][0].height))
            else:
                j = int(rng.integers(0, len(mesh_scenes)))
                plan.append(("mesh", j, mesh_scenes[j][1], 512, 512))
        row = {"requests": n, "arrival_window_s": float(arrivals[-1]) if n else 0.0}
        for mode in ("batched", "plain"):
            ctx = ctx_factory()
            workers = 0 if mode == "plain" else spec_workers
            srv = mm3e_cuda.Server(ctx, hbm_budget_bytes=40 << 30, plain=(mode == "plain"), spec_workers=workers)
            spec_warmup_s = None
            try:
                ids = [srv.add_scene(s) for s, _ in resident]
                if workers:
                    # the resident scenes' kernels compile on host threads while the server starts:
                    # the stream begins once they are loaded (a warm server)
                    t0 = time.perf_counter()
                    while srv.stats()["spec_pending"] > 0 and time.perf_counter() - t0 < 600:
                        time.sleep(0.05)
                    spec_warmup_s = time.perf_counter() - t0
                reqs, keep = [], []
                for kind, j, cam, w, h in plan:
                    out = out_for(w, h)
                    if kind == "resident":
                        r, k = srv.request(cam, out, scene_id=ids[j])
                    elif kind == "new":
                        r, k = srv.request(cam, out, new_scene=fresh[j][0])
                    else:
                        pos, tri = meshes[j]
                        r, k = srv.request(cam, out, new_scene=mesh_scenes[j][0], mesh=(pos, tri), mesh_volume=0,
                                           mesh_resolution=128, mesh_padding=0.1)
                    reqs.append(r)
                    keep.append(k)
                rc, res = srv.replay(reqs, list(arrivals))
                st = srv.stats()
            finally:
                srv.close()
                ctx.close()
            ok = [r for r in res if r["status"] == 0]
            lat = [r["done_ms"] - r["submit_ms"] for r in ok]
            span = (max(r["done_ms"] for r in ok) - min(r["submit_ms"] for r in ok)) / 1000.0 if ok else 0.0
            row[mode] = {"completed": len(ok), "failed": n - len(ok), "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
                         "mean_ms": float(np.mean(lat)) if lat else None,
                         "frames_per_s": len(ok) / span if span > 0 else None,
                         "sequences": st["sequences"], "frames_per_sequence":
                             st["frames_in_sequences"] / max(1, st["sequences"]),
                         "mesh_bakes": st["mesh_bakes"], "scenes_compiled": st["scenes_compiled"],
                         "peak_admitted_bytes": st["peak_admitted_bytes"], "reserved_bytes": st["reserved_bytes"],
                         "spec_workers": workers, "scenes_specialized": st["scenes_specialized"],
                         "spec_frames": st["spec_frames"], "spec_warmup_s": spec_warmup_s}
        if row["batched"]["frames_per_s"] and row["plain"]["frames_per_s"]:
            row["batched_over_plain_frames_per_s"] = row["batched"]["frames_per_s"] / row["plain"]["frames_per_s"]
        results[str(rate)] = row
    return {"workload": "served_poisson", "rates_per_s": list(rates), "hbm_budget_bytes": 40 << 30,
            "arrival_window_s": seconds, "max_requests_per_rate": max_requests, "by_rate": results}


def _tuning(text):
    b, t, u, m = (int(v) for v in text.split(","))
    return {"block": b, "tile_wlog": t, "unroll": u, "min_blocks": m}


def run_profile_frames(args):
    """Renders N frames of the workload through mm3e_render_device and exits (for ncu)."""
    import torch

    import mm3e_cuda
    from mm3e_cuda import abi

    size = tuple(int(v) for v in args.size.lower().split("x")) if args.size else None
    scene, cam = workloads(size)[args.workload]()
    ctx = mm3e_cuda.Context(0)
    compiled = mm3e_cuda.CompiledScene(ctx, scene)
    if not args.no_spec:
        compiled.specialize(compiled.SPEC_AUTO)
    if args.tuning:
        compiled.autotune(cam, spec_mode=0 if args.no_spec else compiled.SPEC_AUTO, candidates=[_tuning(args.tuning)],
                          repeats=1)
    out = torch.empty(scene.width * scene.height * 4, dtype=torch.uint8, device="cuda")
    for _ in range(args.profile_frames):
        compiled.render_device(cam, abi.FB_RGBA8, out.data_ptr(), out.numel())
    ctx.sync()
    print(f"rendered {args.profile_frames} frame(s) of {args.workload} at {scene.width}x{scene.height}"
          f" ({'specialised' if compiled.specialized else 'interpreted'} field)")
    ctx.close()


def load_counts(workload):
    try:
        with open(COUNTS_FIXTURE) as f:
            return json.load(f).get(workload)
    except (OSError, ValueError):
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(k)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload_config(args, scene, world):
    """The `config` dict both arms print (the same workload, the same dict)."""
    return {"workload": args.workload, "width": scene.width, "height": scene.height, "aa": scene.aa,
            "bounces": scene.bounces, "max_steps": scene.marcher.max_steps, "parallelism": f"replicas x{world}",
            "l2": "flushed between timed steps (256 MB write)"}


def cpu_frames(scene, cam, target_s, threads):
    """Whole frames of the workload through the oracle (render + post, all host threads): one
    untimed frame, then frames until about `target_s` seconds are spent (at least one), each
    after a 256 MB host write. Returns (frame seconds list, the last RGBA f32 frame)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import oracle_py

    h = scene.desc()
    flush = np.empty(64 * 1024 * 1024, np.float32)
    t0 = time.perf_counter()
    frame = oracle_py.render(h, cam, threads=threads)
    first = time.perf_counter() - t0
    n = max(1, int(round(target_s / max(first, 1e-3))))
    ts = []
    for i in range(n):
        flush.fill(float(i))
        t0 = time.perf_counter()
        frame = oracle_py.render(h, cam, threads=threads)
        ts.append(time.perf_counter() - t0)
    return ts, frame


def cpu_baseline(scene, cam, target_s):
    """The oracle (CPU restatement of the reference render path) on all host cores, whole frames."""
    threads = os.cpu_count() or 1
    ts, frame = cpu_frames(scene, cam, target_s, threads)
    v = len(ts) / sum(ts)
    return {"value": v, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{len(ts)} whole {scene.width}x{scene.height} frames after one untimed frame "
                      f"(render + post; {sum(ts):.2f} s on {threads} threads)"}, frame


def frame_parity(gpu_rgba8, ref_rgba8, gpu_hits, ref_hits):
    """The parity bars on one frame: (iii) RGB8 within 1 LSB and PSNR; (i) hit/miss and material
    mismatches (silhouettes: pixels with a different id in their 4-neighbourhood); (ii) hit
    distance within 1e-4 relative on agreed hits."""
    import numpy as np

    a = np.asarray(gpu_rgba8)[..., :3].astype(np.int32)
    b = np.asarray(ref_rgba8)[..., :3].astype(np.int32)
    d = np.abs(a - b)
    mse = float((d.astype(np.float64) ** 2).mean())
    out = {"psnr": float("inf") if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse),
           "within1_px": float((d.max(-1) <= 1).mean()), "exact_px": float((d.max(-1) == 0).mean()),
           "max_lsb": int(d.max())}
    gm, rm = gpu_hits["mat"], ref_hits["mat"]
    diff = gm != rm

    def edges(m):
        e = np.zeros(m.shape, bool)
        e[1:, :] |= m[1:, :] != m[:-1, :]
        e[:-1, :] |= m[:-1, :] != m[1:, :]
        e[:, 1:] |= m[:, 1:] != m[:, :-1]
        e[:, :-1] |= m[:, :-1] != m[:, 1:]
        return e

    sil = edges(gm) | edges(rm)
    agreed = (~diff) & (rm != 0xFFFFFFFF)
    rel = np.abs(gpu_hits["t"][agreed].astype(np.float64) - ref_hits["t"][agreed]) / np.maximum(
        np.abs(ref_hits["t"][agreed]), 1e-12)
    out.update({"mismatch_frac": float(diff.mean()), "mismatch_off_silhouette": int((diff & ~sil).sum()),
                "t_within_1e-4": float((rel <= 1e-4).mean()) if rel.size else 1.0,
                "t_rel_max": float(rel.max()) if rel.size else 0.0})
    return out


def run_reference(args):
    """The reference arm: the CPU reference render path (the oracle restatement; the Rust reference
    has no toolchain here) on all host threads, whole frames of the same workload. The scene and
    camera are built through the oracle's own helpers, so libmm3e_cuda.so is never loaded."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import oracle_py
    from mm3e_cuda.scene import use_host_math

    use_host_math(oracle_py.HostMath())
    scene, cam = workloads()[args.workload]()
    threads = os.cpu_count() or 1
    h = scene.desc()
    flush = np.empty(64 * 1024 * 1024, np.float32)
    for _ in range(args.warmup):
        oracle_py.render(h, cam, threads=threads)
    ts = []
    for i in range(args.steps):
        flush.fill(float(i))
        t0 = time.perf_counter()
        oracle_py.render(h, cam, threads=threads)
        ts.append(time.perf_counter() - t0)
    v = len(ts) / sum(ts)
    counts = load_counts(args.workload)
    rays = None
    if counts:
        r = counts["render"]
        rays = (r["primary_rays"] + r["reflection_rays"] + r["shadow_rays"]) * v / 1e6
    cb = {"value": v, "unit": "frames/s", "cores": threads, "kind": "port",
          "sample": f"one whole {scene.width}x{scene.height} frame per step (render + post), all {threads} host "
                    "threads; the CPU restatement of the reference path (oracle/)"}
    print(json.dumps({
        "impl": "reference", "metric": f"frames/s ({args.workload})", "value": v, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(ts) / len(ts),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic seeded scene (no dataset)", "config": workload_config(args, scene, world),
        "mrays_per_s": rays, "cpu_baseline": cb,
        "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def run_ours(args):
    import numpy as np
    import torch

    import mm3e_cuda
    from mm3e_cuda import abi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = mm3e_cuda.Context(local)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    info = ctx.device_info()

    scene, cam = workloads()[args.workload]()
    compiled = mm3e_cuda.CompiledScene(ctx, scene)
    w, h = scene.width, scene.height
    out8 = torch.empty(h * w * 4, dtype=torch.uint8, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2

    fps_step = max(1, args.frames_per_step)

    def frame():
        compiled.render_device(cam, abi.FB_RGBA8, out8.data_ptr(), out8.numel())

    def step():
        for _ in range(fps_step):
            frame()

    def timed(fn, k):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        with torch.cuda.stream(stream):
            for i in range(k):
                flush.fill_(float(i))
                ev[i][0].record(stream)
                fn()
                ev[i][1].record(stream)
        stream.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    # the interpreter first (reported beside), then the scene-specialised kernels the fixed scene
    # renders with (auto policy: small fields only), compiled before the timed region
    for _ in range(max(3, args.warmup)):
        frame()
    interp_ms = timed(frame, max(3, args.steps // 2))
    spec_compile_ms = None
    tuning = None
    if not args.no_spec:
        spec_compile_ms = compiled.specialize(compiled.SPEC_AUTO)
        # the library's own launch-shape search for this scene (specialised kernels recompiled
        # per candidate), before the timed region
        t0 = time.perf_counter()
        best, table = compiled.autotune(cam, spec_mode=compiled.SPEC_AUTO,
                                        candidates=[_tuning(args.tuning)] if args.tuning else None)
        tuning = {"best": best, "table": [[t, round(ms, 3)] for t, ms in table],
                  "search_s": round(time.perf_counter() - t0, 2)}
    specialized = compiled.specialized
    for _ in range(max(3, args.warmup)):
        step()
    stream.synchronize()
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    t0 = time.perf_counter()
    step_ms = timed(step, args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    gpu_frame = out8.view(h, w, 4).cpu().numpy()  # the last timed frame, for the parity check
    frame_ms = [ms / fps_step for ms in step_ms]
    # per-kernel device time: the same frames again with CUDA events around every pass
    ctx.set_profiling(True)
    ctx.kernel_times()
    prof_ms = timed(frame, args.steps)
    kt = ctx.kernel_times()
    ctx.set_profiling(False)

    # e2e: the public call with a host framebuffer (camera in, RGBA8 frame out, every frame),
    # one framebuffer reused across frames as a frame loop would
    host = np.zeros((h, w, 4), np.uint8)
    _, st = compiled.render(cam, fmt=abi.FB_RGBA8, stats=True, out=host)
    launches_per_frame = st["kernel_launches"]
    t1 = time.perf_counter()
    for _ in range(args.steps * fps_step):
        compiled.render(cam, fmt=abi.FB_RGBA8, out=host)
    e2e_s = time.perf_counter() - t1
    clocks = sampler.stop()

    mean_ms = sum(frame_ms) / len(frame_ms)
    if dist:
        t = torch.tensor([mean_ms, e2e_s], device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        mean_ms, e2e_s = float(t[0]), float(t[1])
    if rank != 0:
        ctx.close()
        return

    value = world * 1000.0 / mean_ms
    counts = load_counts(args.workload)
    sm = info["sm_count"]
    max_mhz = clocks.get("sm_max_mhz") or 2070.0
    peak = sm * 128 * 2 * max_mhz * 1e6 / 1e12
    prof_total = sum(ms for _, ms in kt.values())
    kernels = {k: {"launches_per_frame": n / args.steps, "ms_per_frame": ms / args.steps,
                   "share": ms / prof_total if prof_total else None} for k, (n, ms) in kt.items()}
    # the roofline kernel is the primary-level march (the reflection level's event time includes
    # its overlap with the primary level's passes on the other streams)
    dom = "march" if "march" in kt else (max(kt, key=lambda k: kt[k][1]) if kt else "march")
    dom_s = kt[dom][1] / args.steps / 1000.0 if kt else None
    roofline = {"bound": "fp32", "unit": "TFLOP/s", "peak": peak,
                "peak_basis": f"{sm} SMs x 128 FP32 lanes x 2 (FMA) x {max_mhz:.0f} MHz max SM clock "
                              "(nominal; MEASURED_PEAKS.json holds no FP32 figure)",
                "kernel": f"mm3e_spec_{dom}" if specialized and dom in ("march", "shadow", "ao") else f"k_{dom}",
                "kernel_ms_per_frame": None if dom_s is None else dom_s * 1000.0,
                "kernels": kernels, "traffic": None,
                "traffic_basis": "DRAM bytes per primary-level march launch: ncu capture at 960x540 scaled by "
                                 "the pixel ratio",
                "profiled_frame_ms": sum(prof_ms) / len(prof_ms)}
    if args.workload in MARCH_DRAM_BYTES_960x540 and dom == "march":
        roofline["traffic"] = MARCH_DRAM_BYTES_960x540[args.workload] * (w * h) / (960 * 540)
    mrays = None
    if counts:
        r = counts["render"]
        phase = counts.get(dom) or r
        if dom_s:
            roofline["achieved"] = phase["fp32"] / dom_s / 1e12
            roofline["frac"] = roofline["achieved"] / peak
            # the kernels are built with --fmad=false (binary32 parity with the reference), so an
            # FP32 lane retires at most one add or multiply per cycle: half the FMA-counted peak
            roofline["frac_of_unfused_issue_ceiling"] = roofline["achieved"] / (peak / 2.0)
            if clocks.get("sm_mhz"):
                roofline["frac_at_run_clock"] = roofline["achieved"] / (sm * 128 * 2 * clocks["sm_mhz"] * 1e6 / 1e12)
        roofline["algorithmic_fp32_per_frame"] = phase["fp32"]
        roofline["field_evals_per_frame"] = phase["field_evals"]
        roofline["frame_fp32_per_s"] = (r["fp32"] + counts["post"]["fp32"]) * value / 1e12
        rays = r["primary_rays"] + r["reflection_rays"] + r["shadow_rays"]
        mrays = rays * value / 1e6
    cpu, parity = None, None
    if not args.no_cpu:
        cpu, ref_frame = cpu_baseline(scene, cam, args.cpu_seconds)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        parity = frame_parity(gpu_frame, mm3e_cuda.to_rgba8(ref_frame), compiled.render_hits(cam),
                              oracle_py.primary_hits(scene.desc(), cam))
        parity["frame"] = ("the last timed frame (device RGBA8, the timed launch shape) against the oracle's frame "
                           "of the cpu_baseline leg; hits: mm3e_render_hits against the oracle's primary hits")
    e2e_value = world * args.steps * fps_step / e2e_s
    line = {
        "metric": f"frames/s ({args.workload})", "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_ms * fps_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic seeded scene (no dataset)",
        "config": workload_config(args, scene, world),
        "frames_per_step": fps_step,
        "field": "scene-specialised (NVRTC)" if specialized else "tape interpreter",
        "spec_compile_ms": spec_compile_ms, "launch_tuning": tuning,
        "interpreter": {"frames_per_s": 1000.0 / statistics.median(interp_ms),
                        "frame_ms_median": statistics.median(interp_ms)},
        "mrays_per_s": mrays, "frame_ms": {"min": min(frame_ms), "median": statistics.median(frame_ms),
                                           "max": max(frame_ms)},
        "wall_s_timed_region": wall, "roofline": roofline, "cpu_baseline": cpu, "parity": parity,
        "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": 52 * fps_step,
                "d2h_bytes_per_step": w * h * 4 * fps_step},
        "gpu_launches": launches_per_frame * args.steps * fps_step, "clocks": clocks,
    }
    if cpu:
        line["speedup_vs_cpu"] = value / cpu["value"]
        line["e2e_speedup_vs_cpu"] = e2e_value / cpu["value"]
    if not args.no_forms and world == 1:
        line["cornell"] = bench_cornell(ctx, stream, torch)
        line["batched"] = bench_batched(ctx, stream, torch, args.batch_scenes)
        line["preview"] = bench_preview(ctx, torch, not args.no_cpu)
        line["published_scene"] = bench_published(ctx, stream, torch)
        ctx.set_stream(None)
        line["served"] = bench_served(lambda: mm3e_cuda.Context(local), args.served_seconds, args.served_max_requests,
                                      rates=tuple(int(r) for r in args.served_rates.split(",")))
    print(json.dumps(line))
    ctx.close()


def run_served_only(args):
    """Only the served-form measurement (e.g. the full 60 s windows), printed as its own line."""
    import mm3e_cuda

    out = bench_served(lambda: mm3e_cuda.Context(0), args.served_seconds, args.served_max_requests,
                       rates=tuple(int(r) for r in args.served_rates.split(",")))
    print(json.dumps({"served": out}))


def main():
    args = parse()
    if args.served_only:
        run_served_only(args)
    elif args.profile_frames:
        run_profile_frames(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
