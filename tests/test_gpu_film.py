"""render_film on the GPU (mm3e_render_film) against the oracle's render_film and the reference's
film properties (mm3e-orchestrator/tests/film.rs)."""
import json

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from film_scenes import camera, emissive_scene, reflective_scene
from mm3e_cuda import scenes

pytestmark = pytest.mark.gpu


def _compare(name, gpu, ref):
    a, b = gpu["alpha"], ref["alpha"]
    alpha_diff = float((a != b).mean())
    hit = (gpu["material_ids"] != 0xFFFFFFFF) & (gpu["material_ids"] == ref["material_ids"])
    mat_diff = float((gpu["material_ids"] != ref["material_ids"]).mean())
    dd = np.abs(gpu["depth"][hit] - ref["depth"][hit]) / np.maximum(np.abs(ref["depth"][hit]), 1e-6)
    rel = lambda x, y: np.abs(x - y) / np.maximum(np.abs(y), 1e-3)
    beauty_ok = float((rel(gpu["beauty"], ref["beauty"]) <= 1e-3).all(-1).mean())
    fg_ok = float((rel(gpu["foreground"], ref["foreground"]) <= 1e-3).all(-1).mean())
    m = {"alpha_mismatch": alpha_diff, "mat_mismatch": mat_diff, "depth_rel_max": float(dd.max()) if dd.size else 0.0,
         "beauty_within_1e-3": beauty_ok, "foreground_within_1e-3": fg_ok}
    print(name, json.dumps(m))
    assert mat_diff <= 0.001 and m["depth_rel_max"] <= 1e-4, m
    assert alpha_diff <= 0.005 and beauty_ok >= 0.995 and fg_ok >= 0.995, m
    return m


@pytest.mark.parametrize("case", ["reflective_pinhole", "emissive_lens", "gallery_lens", "plane_geometry"])
def test_film_matches_oracle(gpu_ctx, case):
    lens = (0.0, 1.0)
    cam = camera()
    if case == "reflective_pinhole":
        s = reflective_scene()
    elif case == "emissive_lens":
        s, lens = emissive_scene(37, 29, (4.0, 0.6, 0.2)), (0.18, 6.0)
    elif case == "gallery_lens":
        s, cam = scenes.gallery_scene(96, 54)
        s.aa = 3
        lens = (0.25, 11.0)
    else:
        from mm3e_cuda.scene import Object, Prim, Transform
        s = emissive_scene(16, 12, (1.0, 1.0, 1.0))
        s.objects.clear()
        s.add(Object(Prim.plane((0.0, 0.0, 1.0), 0.0), Transform.IDENTITY, 1))
        lens = (0.9, 1.0)
    cs = mm3e_cuda.CompiledScene(gpu_ctx, s)
    gpu = cs.render_film(cam, *lens)
    ref = oracle_py.render_film(s.desc(), cam, *lens)
    _compare(case, gpu, ref)


def test_pinhole_film_beauty_is_the_linear_render(gpu_ctx):
    s = reflective_scene()
    cs = mm3e_cuda.CompiledScene(gpu_ctx, s)
    film = cs.render_film(camera())
    assert np.array_equal(film["beauty"], cs.render_linear(camera()))
    hits = cs.render_hits(camera())
    assert np.array_equal(film["material_ids"], hits["mat"])


def test_film_lens_validation(gpu_ctx):
    cs = mm3e_cuda.CompiledScene(gpu_ctx, emissive_scene(8, 8, (1.0, 1.0, 1.0)))
    for r, f in ((-0.1, 1.0), (float("nan"), 1.0), (0.1, 0.0), (0.1, float("inf"))):
        with pytest.raises(mm3e_cuda.RenderError):
            cs.render_film(camera(), r, f)
