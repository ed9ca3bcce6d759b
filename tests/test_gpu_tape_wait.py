"""Bounded device waits (the reference bounds every loop, march.rs:142,248): the march and shadow
kernels stage the scene tape into shared memory and wait for it on an mbarrier with an iteration
limit. Here the wait is made to run out on purpose: with the probe mode nothing arrives on the
barrier and no tape copy is issued, so the kernels give up after a few iterations with nothing in
flight. The call must report ERR_TIMEOUT, the passes after the failed one must do nothing, and the
next render on the same context must give the exact frame again. All calls go through the C ABI."""
import numpy as np
import pytest

import mm3e_cuda
from mm3e_cuda import abi, scenes

pytestmark = pytest.mark.gpu

LIMIT = 64  # iterations of the staging wait before the kernels give up


def _expect_timeouts(ctx, cs, cam):
    ctx.set_tape_wait(LIMIT, probe=True)
    try:
        for call in (lambda: cs.render(cam, fmt=abi.FB_RGBA8), lambda: cs.render_hits(cam)):
            with pytest.raises(mm3e_cuda.RenderError) as e:
                call()
            assert e.value.code == abi.ERR_TIMEOUT, e.value
            assert "gave up" in e.value.message
    finally:
        ctx.set_tape_wait(0, probe=False)


@pytest.mark.parametrize("spec", [False, True])
def test_tape_wait_gives_up_and_the_context_recovers(gpu_ctx, spec):
    scene, cam = scenes.gallery_scene(160, 90)
    cs = mm3e_cuda.CompiledScene(gpu_ctx, scene)
    if spec:
        cs.specialize(cs.SPEC_ALWAYS)
        assert cs.specialized
    good = cs.render(cam, fmt=abi.FB_RGBA8)
    good_hits = cs.render_hits(cam)
    _expect_timeouts(gpu_ctx, cs, cam)
    assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA8), good)
    again = cs.render_hits(cam)
    assert np.array_equal(again["t"].view(np.uint32), good_hits["t"].view(np.uint32))
    assert np.array_equal(again["mat"], good_hits["mat"])
    # a normal limit set explicitly renders the same frame
    gpu_ctx.set_tape_wait(1 << 20, probe=False)
    try:
        assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA8), good)
    finally:
        gpu_ctx.set_tape_wait(0, probe=False)
    cs.close()


def test_tape_wait_on_a_fresh_scene_fails_cleanly(gpu_ctx):
    """The first render of a scene (pass buffers just allocated, never written) under the probe:
    the passes after the failed march read none of those buffers, and a later render is exact."""
    scene, cam = scenes.spheres_scene(96, 54)
    cs = mm3e_cuda.CompiledScene(gpu_ctx, scene)
    _expect_timeouts(gpu_ctx, cs, cam)
    ref = mm3e_cuda.CompiledScene(gpu_ctx, scene)
    assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA8), ref.render(cam, fmt=abi.FB_RGBA8))
    cs.close()
    ref.close()
