#!/usr/bin/env python
"""Benchmark of the GB300 per-pixel SDF render path (one JSON line on rank 0).

Workload (default): the 1080p feature gallery (1920x1080, aa 1, one reflection bounce, soft
shadows, AO, fog, sky IBL, bloom + ACES; 11 primitives, smooth union, twist/bend/onion/round/
repeat/mirror; max 256 steps). A step = one frame rendered on the GPU from the resident
scene tape to a device RGBA8 framebuffer (render kernel + post kernels).

  value      frames/s with the scene resident in HBM (CUDA events on the render stream,
             L2 flushed between timed frames by writing a 256 MB buffer)
  e2e        frames/s through the public C ABI call mm3e_render with a host framebuffer:
             per frame the camera goes host->device and the RGBA8 frame device->host
  roofline   FP32-pipe roofline of the dominant kernel (the march tape interpreter): the
             algorithmic f32 operations of its phase per frame (oracle operation count split by
             kernel, committed fixture) / its CUDA-event-timed device time per frame (events
             around every pass, a second run of the same frames), against SMs x 128 lanes x 2 x
             max SM clock
  cpu_baseline  the CPU restatement of the reference render path on all host cores, timed on
             a bounded row sample (rows scaled to a full frame) plus its single-thread post pass

--impl reference times the CPU reference path (the oracle restatement: the Rust reference has no
toolchain here) on the same workload and prints its own line. Multi-GPU runs are replicas:
each rank renders its own frames (scaling "weak").
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "atom-3d-engine_gb300"))

COUNTS_FIXTURE = os.path.join(ROOT, "tests", "golden", "workload_counts.json")


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
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="gallery_1080p")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline sample time")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="only render this many frames of the workload (no timing, no JSON line): the "
                         "command profilers run")
    ap.add_argument("--size", default=None, help="WxH resolution override (with --profile-frames)")
    return ap.parse_args()


def run_profile_frames(args):
    """Renders N frames of the workload through mm3e_render_device and exits (for ncu)."""
    import torch

    import mm3e_cuda
    from mm3e_cuda import abi

    size = tuple(int(v) for v in args.size.lower().split("x")) if args.size else None
    scene, cam = workloads(size)[args.workload]()
    ctx = mm3e_cuda.Context(0)
    compiled = mm3e_cuda.CompiledScene(ctx, scene)
    out = torch.empty(scene.width * scene.height * 4, dtype=torch.uint8, device="cuda")
    for _ in range(args.profile_frames):
        compiled.render_device(cam, abi.FB_RGBA8, out.data_ptr(), out.numel())
    ctx.sync()
    print(f"rendered {args.profile_frames} frame(s) of {args.workload} at {scene.width}x{scene.height}")
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


def cpu_baseline(scene, cam, target_s):
    """Oracle render of a bounded row sample on all host cores + its post pass, scaled to a frame."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import oracle_py

    threads = os.cpu_count() or 1
    h = scene.desc()
    probe_rows = max(4, scene.height // 64)
    y0 = scene.height // 2 - probe_rows // 2
    t_probe = oracle_py.time_rows(h, cam, y0, y0 + probe_rows, threads)
    rows = int(min(scene.height, max(probe_rows, probe_rows * target_s / max(t_probe, 1e-3))))
    y0 = max(0, scene.height // 2 - rows // 2)
    # rows centred on the frame's middle band, where the scene content (and the cost) sits
    t_rows = oracle_py.time_rows(h, cam, y0, y0 + rows, threads)
    hdr = np.zeros((scene.height, scene.width, 3), np.float32)
    hdr[y0:y0 + rows] = oracle_py.render_rows(h, cam, y0, y0 + rows, threads)
    t0 = time.perf_counter()
    oracle_py.post(h, hdr)
    t_post = time.perf_counter() - t0
    frame_s = t_rows * scene.height / rows + t_post
    return {"value": 1.0 / frame_s, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"rows {y0}-{y0 + rows} of {scene.height} ({t_rows:.2f} s on {threads} threads, scaled "
                      f"to the frame) + full-frame post pass ({t_post:.2f} s, single thread as post::resolve)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene, cam = workloads()[args.workload]()
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_baseline(scene, cam, per_step)
    vals = [cpu_baseline(scene, cam, per_step) for _ in range(args.steps)]
    v = statistics.median([x["value"] for x in vals])
    cb = dict(vals[0])
    cb["value"] = v
    counts = load_counts(args.workload)
    rays = None
    if counts:
        r = counts["render"]
        rays = (r["primary_rays"] + r["reflection_rays"] + r["shadow_rays"]) * v / 1e6
    print(json.dumps({
        "impl": "reference", "metric": f"frames/s ({args.workload})", "value": v, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic seeded scene", "config": {"workload": args.workload, "width": scene.width,
                                                     "height": scene.height, "aa": scene.aa},
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
    hdr = torch.empty(h * w * 4, dtype=torch.float32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2

    def frame():
        compiled.render_device(cam, abi.FB_RGBA8, out8.data_ptr(), out8.numel())

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

    for _ in range(max(3, args.warmup)):
        frame()
    stream.synchronize()
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    t0 = time.perf_counter()
    frame_ms = timed(frame, args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    # per-kernel device time: the same frames again with CUDA events around every pass
    ctx.set_profiling(True)
    ctx.kernel_times()
    prof_ms = timed(frame, args.steps)
    kt = ctx.kernel_times()
    ctx.set_profiling(False)

    # e2e: the public call with a host framebuffer (camera in, RGBA8 frame out, every frame)
    host = np.empty((h, w, 4), np.uint8)
    _, st = compiled.render(cam, fmt=abi.FB_RGBA8, stats=True)
    launches_per_frame = st["kernel_launches"]
    t1 = time.perf_counter()
    for _ in range(args.steps):
        host = compiled.render(cam, fmt=abi.FB_RGBA8)
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
    dom = max(kt, key=lambda k: kt[k][1]) if kt else "march"
    dom_s = kt[dom][1] / args.steps / 1000.0 if kt else None
    roofline = {"bound": "fp32", "unit": "TFLOP/s", "peak": peak,
                "peak_basis": f"{sm} SMs x 128 FP32 lanes x 2 (FMA) x {max_mhz:.0f} MHz max SM clock "
                              "(nominal; MEASURED_PEAKS.json holds no FP32 figure)",
                "kernel": f"k_{dom}", "kernel_ms_per_frame": None if dom_s is None else dom_s * 1000.0,
                "kernels": kernels, "traffic": None,
                "profiled_frame_ms": sum(prof_ms) / len(prof_ms)}
    mrays = None
    if counts:
        r = counts["render"]
        phase = counts.get(dom) or r
        if dom_s:
            roofline["achieved"] = phase["fp32"] / dom_s / 1e12
            roofline["frac"] = roofline["achieved"] / peak
            if clocks.get("sm_mhz"):
                roofline["frac_at_run_clock"] = roofline["achieved"] / (sm * 128 * 2 * clocks["sm_mhz"] * 1e6 / 1e12)
        roofline["algorithmic_fp32_per_frame"] = phase["fp32"]
        roofline["field_evals_per_frame"] = phase["field_evals"]
        roofline["frame_fp32_per_s"] = (r["fp32"] + counts["post"]["fp32"]) * value / 1e12
        rays = r["primary_rays"] + r["reflection_rays"] + r["shadow_rays"]
        mrays = rays * value / 1e6
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(scene, cam, args.cpu_seconds)
    e2e_value = world * args.steps / e2e_s
    line = {
        "metric": f"frames/s ({args.workload})", "value": value, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic seeded scene (no dataset)",
        "config": {"workload": args.workload, "width": w, "height": h, "aa": scene.aa, "bounces": scene.bounces,
                   "max_steps": scene.marcher.max_steps, "parallelism": f"replicas x{world}",
                   "l2": "flushed between timed frames (256 MB write)"},
        "mrays_per_s": mrays, "frame_ms": {"min": min(frame_ms), "median": statistics.median(frame_ms),
                                           "max": max(frame_ms)},
        "wall_s_timed_region": wall, "roofline": roofline, "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": 52, "d2h_bytes_per_step": w * h * 4},
        "gpu_launches": launches_per_frame * args.steps, "clocks": clocks,
    }
    if cpu:
        line["speedup_vs_cpu"] = value / cpu["value"]
        line["e2e_speedup_vs_cpu"] = e2e_value / cpu["value"]
    print(json.dumps(line))
    ctx.close()


def main():
    args = parse()
    if args.profile_frames:
        run_profile_frames(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
