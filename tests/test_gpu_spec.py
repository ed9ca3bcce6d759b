"""Scene-specialised kernels (NVRTC): frames and hit records identical to the interpreter's.

The specialised field calls the library's own object code on constant copies of the scene's
records and folds the world plan exactly as the interpreter does, so the two paths agree bit for
bit; the interpreter itself is checked against the CPU oracle in test_gpu_parity.py.
"""
import numpy as np
import pytest

import mm3e_cuda
from mm3e_cuda import abi, scenes
from field_scenes import csg_zoo_scene, noncons_scene, planes_scene, smooth_chain_scene, unbounded_mix_scene
from mm3e_cuda.scene import DynSphere

pytestmark = pytest.mark.gpu

SCENES = {
    "spheres": lambda: scenes.spheres_scene(160, 90),
    "gallery": lambda: scenes.gallery_scene(192, 108),
    "hero_aa2_b2": lambda: scenes.hero_scene(120, 68, 2, 2),
    "demo": scenes.demo_scene,
    "canonical_assets": scenes.canonical_asset_scene,
    "procedural0": lambda: scenes.procedural_scene(0, 96, 64),
    "procedural4": lambda: scenes.procedural_scene(4, 96, 64),
    "noncons": lambda: noncons_scene(21, 160, 90),
    "smooth_chain": lambda: smooth_chain_scene(5, 160, 90),
    "csg_zoo1": lambda: csg_zoo_scene(1, 160, 90),
    "csg_zoo3": lambda: csg_zoo_scene(3, 160, 90),
    "procedural9": lambda: scenes.procedural_scene(9, 128, 72),
    "planes": lambda: planes_scene(160, 90),
    "unbounded_mix": lambda: unbounded_mix_scene(4, 160, 90),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_specialised_equals_interpreted(gpu_ctx, name):
    scene, cam = SCENES[name]()
    cs = mm3e_cuda.CompiledScene(gpu_ctx, scene)
    ref8 = cs.render(cam, fmt=abi.FB_RGBA8)
    ref32 = cs.render(cam, fmt=abi.FB_RGBA_F32)
    hits = cs.render_hits(cam)
    ms = cs.specialize()
    print(name, "compile ms", round(ms))
    assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA8), ref8)
    assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA_F32), ref32)
    h2 = cs.render_hits(cam)
    for k in ("t", "mat", "steps", "normal"):
        assert np.array_equal(h2[k], hits[k]), k
    cs.specialize(False)
    assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA8), ref8)


def test_specialised_scene_with_dynamic_spheres_uses_the_interpreter(gpu_ctx):
    scene, cam = scenes.spheres_scene(96, 54)
    cs = mm3e_cuda.CompiledScene(gpu_ctx, scene)
    dyn = [DynSphere((0.5, 0.6, -1.0), 0.4, (0.9, 0.3, 0.2), 0.0)]
    ref = cs.render(cam, dyn_spheres=dyn, fmt=abi.FB_RGBA8)
    cs.specialize()
    assert np.array_equal(cs.render(cam, dyn_spheres=dyn, fmt=abi.FB_RGBA8), ref)


def test_auto_mode_keeps_the_interpreter_for_large_fields(gpu_ctx):
    from mm3e_cuda.scene import Object, Prim, Transform

    big, cam = scenes.procedural_scene(4, 64, 48)  # 62 objects, plus spheres past the 64 limit
    for k in range(8):
        big.add(Object(Prim.sphere(0.2), Transform.at((8.0 + k, 0.5, 8.0)), 0))
    cs = mm3e_cuda.CompiledScene(gpu_ctx, big)
    cs.specialize(cs.SPEC_AUTO)
    assert not cs.specialized
    small, cam2 = scenes.gallery_scene(64, 36)
    cs2 = mm3e_cuda.CompiledScene(gpu_ctx, small)
    cs2.specialize(cs2.SPEC_AUTO)
    assert cs2.specialized


def test_scene_autotune_keeps_frames(gpu_ctx):
    """mm3e_scene_autotune times candidate launch shapes and keeps the fastest as the scene's own;
    frames are identical under every shape."""
    scene, cam = scenes.gallery_scene(192, 108)
    cs = mm3e_cuda.CompiledScene(gpu_ctx, scene)
    ref = cs.render(cam, fmt=abi.FB_RGBA8)
    cands = [{"block": 128, "tile_wlog": 3, "unroll": 1, "min_blocks": 0},
             {"block": 256, "tile_wlog": 4, "unroll": 1, "min_blocks": 0},
             {"block": 128, "tile_wlog": 2, "unroll": 2, "min_blocks": 8}]
    best, table = cs.autotune(cam, spec_mode=cs.SPEC_ALWAYS, candidates=cands, repeats=2)
    print("autotune", best, table)
    assert len(table) == 3 and best in [t for t, _ in table]
    assert cs.specialized
    assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA8), ref)
    assert gpu_ctx.get_tuning()["block"] == 128  # the context's own tuning is untouched
