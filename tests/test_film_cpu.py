"""render_film on the oracle, against the reference's own film tests
(mm3e-orchestrator/tests/film.rs:29-170)."""
import numpy as np
import pytest

import oracle_py
from film_scenes import camera, emissive_scene, reflective_scene
from mm3e_cuda.scene import Object, Prim, Transform


def test_pinhole_beauty_is_bitwise_canonical():
    s = reflective_scene()
    film = oracle_py.render_film(s.desc(), camera())
    _, hdr = oracle_py.render(s.desc(), camera(), want_hdr=True)
    assert np.array_equal(film["beauty"], hdr)
    again = oracle_py.render_film(s.desc(), camera(), threads=1)
    for k in film:
        assert np.array_equal(film[k], again[k]), k


def test_premultiplied_foreground_composites_over_a_physical_background():
    emission = np.array([4.0, 0.6, 0.2], np.float32)
    s = emissive_scene(37, 29, tuple(emission))
    film = oracle_py.render_film(s.desc(), camera(), 0.18, 6.0)
    a = film["alpha"]
    assert ((a > 0) & (a < 1)).any() and (a == 0).any() and (a == 1).any()
    background = np.array([0.02, 0.08, 0.3], np.float32)
    ref = emissive_scene(37, 29, tuple(emission))
    from mm3e_cuda.scene import Material
    m = ref.material(Material(albedo=(0.0, 0.0, 0.0), emissive=tuple(background)))
    ref.add(Object(Prim.plane((0.0, 0.0, 1.0), 3.0), Transform.IDENTITY, m))
    physical = oracle_py.render_film(ref.desc(), camera(), 0.18, 6.0, threads=1)
    assert np.abs(film["foreground"] - emission * a[..., None]).max() < 1e-6
    comp = film["foreground"] + background * (1.0 - a[..., None])
    assert np.linalg.norm(comp - physical["beauty"], axis=-1).max() < 3e-6
    assert (film["foreground"][a == 0] == 0).all()


def test_black_geometry_is_opaque_and_primary_sky_is_uncovered():
    s = emissive_scene(13, 13, (0.0, 0.0, 0.0))
    film = oracle_py.render_film(s.desc(), camera())
    assert film["alpha"][6, 6] == 1.0
    assert (film["foreground"][6, 6] == 0).all() and (film["beauty"][6, 6] == 0).all()
    assert film["alpha"][0, 0] == 0.0
    assert np.linalg.norm(film["beauty"][0, 0]) > 0.1
    assert film["depth"][0, 0] == np.inf
    assert (film["normals"][0, 0] == 0).all()
    assert film["material_ids"][0, 0] == 0xFFFFFFFF


def test_geometry_passes_are_raw_centre_pinhole():
    s = emissive_scene(3, 3, (1.0, 1.0, 1.0))
    s.objects.clear()
    s.add(Object(Prim.plane((0.0, 0.0, 1.0), 0.0), Transform.IDENTITY, 1))
    film = oracle_py.render_film(s.desc(), camera(), 0.9, 1.0)
    assert np.abs(film["depth"] - 3.0).max() < 1e-4
    assert np.linalg.norm(film["normals"] - np.array([0, 0, 1.0]), axis=-1).max() < 1e-5
    assert (film["material_ids"] == 1).all()
    sphere = oracle_py.render_film(emissive_scene(3, 3, (1.0, 1.0, 1.0)).desc(), camera(), 0.9, 1.0)
    assert abs(sphere["depth"][1, 1] - 2.45) < 1e-4


def test_aperture_changes_coverage_but_not_geometry():
    s = emissive_scene(31, 25, (1.0, 1.0, 1.0))
    s.aa = 6
    pin = oracle_py.render_film(s.desc(), camera())
    ap = oracle_py.render_film(s.desc(), camera(), 0.3, 7.0)
    ap8 = oracle_py.render_film(s.desc(), camera(), 0.3, 7.0, threads=8)
    for k in ap:
        assert np.array_equal(ap[k], ap8[k]), k
    assert not np.array_equal(pin["alpha"], ap["alpha"])
    for k in ("depth", "normals", "material_ids"):
        assert np.array_equal(pin[k], ap[k]), k
    part = lambda a: int(((a > 0) & (a < 1)).sum())
    assert part(ap["alpha"]) > part(pin["alpha"])


@pytest.mark.parametrize("radius,focus", [(-0.1, 1.0), (float("nan"), 1.0), (float("inf"), 1.0), (0.1, 0.0),
                                          (0.1, -1.0), (0.1, float("nan")), (0.1, float("inf"))])
def test_lens_validation(radius, focus):
    with pytest.raises(ValueError):
        oracle_py.render_film(emissive_scene(4, 4, (1.0, 1.0, 1.0)).desc(), camera(), radius, focus)
