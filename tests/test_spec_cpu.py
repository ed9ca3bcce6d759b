"""Scene-specialised programs on the host: generated for every kind of scene and compiled by
NVRTC to an sm_103a cubin (no device needed; skipped where NVRTC is not installed)."""
import pytest

import mm3e_cuda
from mm3e_cuda import scenes


def test_generated_program_names_every_segment():
    s, _ = scenes.gallery_scene(32, 18)
    src = mm3e_cuda.spec_source(s)
    assert "mm3e_spec_march" in src and "mm3e_spec_shadow" in src and "mm3e_spec_ao" in src
    assert "// segment 0" in src
    assert src.count("__device__ __forceinline__ Field obj_") >= 10


@pytest.mark.parametrize("name", ["spheres", "gallery", "canonical_assets"])
def test_generated_program_compiles(name):
    s, _ = {"spheres": lambda: scenes.spheres_scene(32, 18), "gallery": lambda: scenes.gallery_scene(32, 18),
            "canonical_assets": scenes.canonical_asset_scene}[name]()
    ok, msg, ms = mm3e_cuda.spec_compile_check(s)
    if not ok and "libnvrtc not found" in msg:
        pytest.skip("NVRTC is not installed")
    assert ok, msg


@pytest.mark.parametrize("name", ["smooth_chain", "noncons", "procedural2"])
def test_generated_program_compiles_with_every_cull(name):
    """Programs that use the squared weak-bound test, the non-conservative pre-test, and the
    union / smooth-union / subtraction segment skips compile too."""
    from field_scenes import noncons_scene, smooth_chain_scene

    s, _ = {"smooth_chain": lambda: smooth_chain_scene(5, 32, 18), "noncons": lambda: noncons_scene(21, 32, 18),
            "procedural2": lambda: scenes.procedural_scene(2, 32, 18)}[name]()
    src = mm3e_cuda.spec_source(s)
    if name == "smooth_chain":
        assert "__fadd_ru(acc.d, " in src and "fmaxf(-acc.d, " in src
    if name == "noncons":
        assert "far_beyond(d2, fmaxf(bd, " in src
    ok, msg, ms = mm3e_cuda.spec_compile_check(s)
    if not ok and "libnvrtc not found" in msg:
        pytest.skip("NVRTC is not installed")
    assert ok, msg
