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
        assert "far_beyond_lin_pos(dist2_below(p, CB, " in src and "fmaxf(bd, " in src
    ok, msg, ms = mm3e_cuda.spec_compile_check(s)
    if not ok and "libnvrtc not found" in msg:
        pytest.skip("NVRTC is not installed")
    assert ok, msg


def test_plain_sphere_members_only_where_the_bound_is_the_field():
    """Only a sphere with the identity rotation, unit scale and no modifiers takes its bound
    distance as its exact field; scaled, rotated or rounded spheres keep their own evaluation."""
    from mm3e_cuda.scene import Material, Object, Prim, Scene, Transform, mat3_from_euler

    def count(obj):
        s = Scene(16, 16)
        s.materials = [Material((0.8, 0.8, 0.8))]
        s.objects = [Object(Prim.plane((0.0, 1.0, 0.0), 0.0), Transform.IDENTITY, 0), obj,
                     Object(Prim.sphere(0.3), Transform((9.0, 1.0, 9.0)), 0)]
        return mm3e_cuda.spec_source(s).count("its exact field is its bound distance")

    plain = Object(Prim.sphere(0.7), Transform((0.5, 1.0, -0.25)), 0)
    assert count(plain) == 2
    assert count(Object(Prim.sphere(0.7), Transform((0.5, 1.0, -0.25), scale=2.0), 0)) == 1
    assert count(Object(Prim.sphere(0.7), Transform((0.5, 1.0, -0.25), mat3_from_euler(0.1, 0.2, 0.3)), 0)) == 1
    assert count(plain.round(0.05)) == 1
    assert count(Object(Prim.box((0.5, 0.5, 0.5)), Transform((0.5, 1.0, -0.25)), 0)) == 1


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_csg_programs_are_generated_code(seed):
    """Every CSG object's program (csg.rs:95-118) becomes straight-line code in the specialised
    field: no call of the stack interpreter remains, each object gets its own program, and the
    program compiles."""
    from field_scenes import csg_zoo_scene

    s, _ = csg_zoo_scene(seed, 32, 18)
    src = mm3e_cuda.spec_source(s)
    n_csg = sum(1 for o in s.objects if o.prim.kind == 11)
    assert n_csg == 10
    assert "csg_eval" not in src
    assert src.count("__device__ __forceinline__ float csg_") == n_csg
    ok, msg, ms = mm3e_cuda.spec_compile_check(s)
    if not ok and "libnvrtc not found" in msg:
        pytest.skip("NVRTC is not installed")
    assert ok, msg


def test_axis_planes_are_one_addition():
    """Planes whose normal is an axis (+0 elsewhere), with the identity rotation and an offset
    other than -0, are generated as one addition; the tilted plane and the -0 offset keep the
    general field. The bit-identity with the interpreter is checked on the GPU
    (test_gpu_spec.py, planes)."""
    from field_scenes import planes_scene

    s, _ = planes_scene(32, 18)
    src = mm3e_cuda.spec_source(s)
    assert src.count("// axis plane") == 4
    ok, msg, ms = mm3e_cuda.spec_compile_check(s)
    if not ok and "libnvrtc not found" in msg:
        pytest.skip("NVRTC is not installed")
    assert ok, msg
