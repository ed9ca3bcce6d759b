"""Regenerate the committed fixtures under tests/golden/ from the CPU oracle.

  python tests/golden/make_fixtures.py

* workload_counts.json  algorithmic work per frame of the benchmark workloads (the oracle's
                        counting instantiation: f32 ops, field evaluations, rays), render and
                        post phases and the render phase split by kernel and level (march,
                        ao, shadow, shade, march_refl, ao_refl, shadow_refl); bench.py reads
                        it for Mrays/s and the roofline.
* oracle_frames.npz     small RGB8 frames of the parity scenes rendered by the oracle; the CPU
                        suite checks the oracle still reproduces them bit-exactly and the GPU
                        suite compares the CUDA path against them.
* reference_images.json agreement of the oracle with the images the reference repository
                        ships (its own renders of its example scenes), when its checkout is
                        given in the environment variable MM3E_REFERENCE_DIR.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "atom-3d-engine_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mm3e_cuda  # noqa: E402
import oracle_py  # noqa: E402
from mm3e_cuda import scenes  # noqa: E402
from mm3e_cuda.scene import GiVolume  # noqa: E402

# A checkout of the reference repository (its shipped PNG renders), if any.
REFERENCE = os.environ.get("MM3E_REFERENCE_DIR", "")


def desc_digest(scene):
    """Digest of the scene description bytes (objects, materials, lights, settings)."""
    h = scene.desc()
    d = h.desc
    m = hashlib.sha256()
    import ctypes as C
    m.update(bytes(d)[:C.sizeof(d)])
    for arr, n in ((d.objects, d.n_objects), (d.materials, d.n_materials), (d.lights, d.n_lights)):
        if n:
            m.update(C.string_at(arr, n * C.sizeof(arr._type_)))
    return m.hexdigest()[:16]


def counts():
    from bench import workloads
    out = {}
    for name, fn in workloads().items():
        s, cam = fn()
        c = oracle_py.count_frame(s.desc(), cam)
        c["digest"] = desc_digest(s)
        out[name] = c
        print(name, c["render"]["fp32"], c["render"]["field_evals"])
    return out


def parity_scenes():
    return {
        "spheres_160x90": lambda: scenes.spheres_scene(160, 90),
        "gallery_160x90": lambda: scenes.gallery_scene(160, 90),
        "hero_120x68_aa2": lambda: scenes.hero_scene(120, 68, 2, 2),
        "demo_96x64": scenes.demo_scene,
        "canonical_assets_65x41": scenes.canonical_asset_scene,
        "procedural0_128x72": lambda: scenes.procedural_scene(0, 128, 72),
    }


def frames():
    out = {}
    for name, fn in parity_scenes().items():
        s, cam = fn()
        out[name] = mm3e_cuda.to_rgba8(oracle_py.render(s.desc(), cam, threads=1))[..., :3]
    return out


def reference_images():
    res = {}
    if not REFERENCE or not os.path.isdir(REFERENCE):
        return res
    from tests_png import read_png
    for fname, fn, bake in (("spheres.png", lambda: scenes.hero_scene(960, 540, 2, 2), None),
                            ("gallery.png", scenes.reference_gallery_scene, None),
                            ("gi_demo.png", scenes.reference_gi_demo_scene, ((20, 14, 20), 5))):
        path = os.path.join(REFERENCE, fname)
        if not os.path.exists(path):
            continue
        s, cam = fn()
        if bake:
            g = oracle_py.bake_gi(s.desc(), *bake)
            s.gi = GiVolume(*g)
        ours = mm3e_cuda.to_rgba8(oracle_py.render(s.desc(), cam))[..., :3].astype(np.int32)
        ref = read_png(path)[..., :3].astype(np.int32)
        d = np.abs(ours - ref).max(-1)
        mse = float(((ours - ref).astype(np.float64) ** 2).mean())
        res[fname] = {"exact_px": float((d == 0).mean()), "within1_px": float((d <= 1).mean()),
                      "psnr_db": 10 * np.log10(255 ** 2 / mse) if mse else float("inf")}
        print(fname, res[fname])
    return res


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    sys.path.insert(0, HERE)
    with open(os.path.join(HERE, "workload_counts.json"), "w") as f:
        json.dump(counts(), f, indent=1)
    if "--counts-only" in sys.argv:
        sys.exit(0)
    np.savez_compressed(os.path.join(HERE, "oracle_frames.npz"), **frames())
    ri = reference_images()
    if ri:
        with open(os.path.join(HERE, "reference_images.json"), "w") as f:
            json.dump(ri, f, indent=1)
