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
