"""Batched form: many scenes, cameras and resolutions per pass sequence (mm3e_render_batch).

A batched frame must be byte-identical to the plain per-frame call of the same scene and camera
at the same size: the batch runs the same kernels over a device job table, with each lane
reading its own job's tape. The plain call is itself checked against the CPU oracle
(test_gpu_parity.py), so equality here carries the oracle parity over to the batched form.
"""
import numpy as np
import pytest

import mm3e_cuda
from mm3e_cuda import abi, scenes
from mm3e_cuda.scene import Scene

pytestmark = pytest.mark.gpu


def _mixed(ctx, sizes):
    """Compiled scenes of different kinds, each with a camera and a render size."""
    out = []
    for k, (w, h) in enumerate(sizes):
        if k % 4 == 0:
            s, cam = scenes.gallery_scene(w, h)
        elif k % 4 == 1:
            s, cam = scenes.spheres_scene(w, h)
        elif k % 4 == 2:
            s, cam = scenes.hero_scene(w, h, 2, 1)
        else:
            s, cam = scenes.procedural_scene(k, w, h)
        out.append((mm3e_cuda.CompiledScene(ctx, s), cam, w, h))
    return out


def _plain(cs, cam):
    return cs.render(cam, fmt=abi.FB_RGBA8)


def test_batch_equals_plain_frames_host_outputs():
    ctx = mm3e_cuda.Context(0)
    try:
        items = _mixed(ctx, [(96, 54), (64, 64), (80, 45), (72, 40), (33, 17), (128, 72), (50, 50), (31, 29)])
        outs = [np.zeros((h, w, 4), np.uint8) for _, _, w, h in items]
        jobs = ctx.make_jobs([(cs, cam, 0, 0, abi.FB_RGBA8, None, o) for (cs, cam, _, _), o in zip(items, outs)])
        st = ctx.render_batch(jobs)
        assert st["sequences"] >= 1 and st["kernel_launches"] > 0
        for (cs, cam, w, h), o in zip(items, outs):
            ref = _plain(cs, cam)
            assert np.array_equal(o, ref), f"batched frame differs from the plain frame ({w}x{h})"
    finally:
        ctx.close()


def test_batch_without_ao_samples_equals_plain_frames():
    """A batch whose only AO scene has no AO samples runs no AO pass; its frames shade with AO 1,
    as the plain frames do (and the oracle, test_gpu_parity.py)."""
    ctx = mm3e_cuda.Context(0)
    try:
        items = []
        for k, (w, h) in enumerate([(64, 36), (40, 30), (33, 17)]):
            s, cam = scenes.gallery_scene(w, h) if k != 1 else scenes.procedural_scene(5, w, h)
            s.marcher.ao_samples = 0
            items.append((mm3e_cuda.CompiledScene(ctx, s), cam, w, h))
        outs = [np.zeros((h, w, 4), np.uint8) for _, _, w, h in items]
        jobs = ctx.make_jobs([(cs, cam, 0, 0, abi.FB_RGBA8, None, o) for (cs, cam, _, _), o in zip(items, outs)])
        ctx.render_batch(jobs)
        for (cs, cam, w, h), o in zip(items, outs):
            assert np.array_equal(o, _plain(cs, cam)), f"batched frame differs from the plain frame ({w}x{h})"
    finally:
        ctx.close()


def test_batch_device_outputs_graphs_and_small_waves():
    torch = pytest.importorskip("torch")
    ctx = mm3e_cuda.Context(0)
    try:
        items = _mixed(ctx, [(64, 36), (48, 48), (40, 30), (56, 32), (20, 12), (90, 50)])
        refs = [_plain(cs, cam) for cs, cam, _, _ in items]
        for use_graphs in (True, False):
            for max_samples in (0, 6000):  # 6000 samples forces several pass sequences
                ctx.configure_batch(max_samples=max_samples, use_graphs=use_graphs)
                bufs = [torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda") for _, _, w, h in items]
                jobs = ctx.make_jobs([(cs, cam, 0, 0, abi.FB_RGBA8, b.data_ptr(), None)
                                      for (cs, cam, _, _), b in zip(items, bufs)])
                st = ctx.render_batch(jobs)
                if max_samples:
                    assert st["sequences"] > 1
                if use_graphs:
                    assert st["graph_launches"] == st["sequences"]
                for (cs, cam, w, h), b, ref in zip(items, bufs, refs):
                    got = b.cpu().numpy().reshape(h, w, 4)
                    assert np.array_equal(got, ref), f"graphs={use_graphs} max_samples={max_samples}: {w}x{h} differs"
    finally:
        ctx.close()


def test_batch_tiny_frames_and_wide_bloom():
    """Jobs of one pixel, one row or one column, and bloom kernels wider than their frames, packed
    next to each other: the post stack's blur windows then span several jobs, and every tap must
    stay in its own job's row or column."""
    ctx = mm3e_cuda.Context(0)
    try:
        items = []
        for k, (w, h, r) in enumerate([(1, 1, 12), (9, 1, 40), (1, 9, 12), (13, 7, 1), (70, 3, 33), (5, 5, 0),
                                       (2, 31, 32), (300, 2, 12)]):
            s, cam = scenes.gallery_scene(w, h) if k % 2 == 0 else scenes.hero_scene(w, h, 2, 1)
            s.post.bloom_radius = r
            items.append((mm3e_cuda.CompiledScene(ctx, s), cam, w, h))
        outs = [np.zeros((h, w, 4), np.uint8) for _, _, w, h in items]
        jobs = ctx.make_jobs([(cs, cam, 0, 0, abi.FB_RGBA8, None, o) for (cs, cam, _, _), o in zip(items, outs)])
        ctx.render_batch(jobs)
        for (cs, cam, w, h), o in zip(items, outs):
            assert np.array_equal(o, _plain(cs, cam)), f"batched frame differs from the plain frame ({w}x{h})"
    finally:
        ctx.close()


def test_batch_resolution_override_matches_scene_compiled_at_that_size():
    ctx = mm3e_cuda.Context(0)
    try:
        s_small, cam = scenes.gallery_scene(40, 24)
        s_big, _ = scenes.gallery_scene(120, 68)
        cs_small = mm3e_cuda.CompiledScene(ctx, s_small)
        cs_big = mm3e_cuda.CompiledScene(ctx, s_big)
        out = np.zeros((68, 120, 4), np.uint8)
        jobs = ctx.make_jobs([(cs_small, cam, 120, 68, abi.FB_RGBA8, None, out)])
        ctx.render_batch(jobs)
        assert np.array_equal(out, cs_big.render(cam, fmt=abi.FB_RGBA8))
    finally:
        ctx.close()


def test_batch_f32_output_and_tile_shapes():
    ctx = mm3e_cuda.Context(0)
    try:
        items = _mixed(ctx, [(50, 30), (37, 21), (64, 40), (45, 45)])
        refs = [cs.render(cam, fmt=abi.FB_RGBA_F32) for cs, cam, _, _ in items]
        for block, wlog, unroll in ((128, 3, 1), (256, 2, 16), (128, 4, 64), (256, 5, 1)):
            ctx.set_tuning(block, wlog, unroll)
            outs = [np.zeros((h, w, 4), np.float32) for _, _, w, h in items]
            jobs = ctx.make_jobs([(cs, cam, 0, 0, abi.FB_RGBA_F32, None, o) for (cs, cam, _, _), o in zip(items, outs)])
            ctx.render_batch(jobs)
            for (cs, cam, w, h), o, ref in zip(items, outs, refs):
                assert np.array_equal(o, ref), f"tuning {block}/{wlog}/{unroll}: {w}x{h} differs"
                # the plain path under the same tuning gives the same frame too
                assert np.array_equal(cs.render(cam, fmt=abi.FB_RGBA_F32), ref)
    finally:
        ctx.close()


def test_autotune_picks_a_listed_shape():
    ctx = mm3e_cuda.Context(0)
    try:
        items = _mixed(ctx, [(64, 36), (48, 48)])
        outs = [np.zeros((h, w, 4), np.uint8) for _, _, w, h in items]
        jobs = ctx.make_jobs([(cs, cam, 0, 0, abi.FB_RGBA8, None, o) for (cs, cam, _, _), o in zip(items, outs)])
        best, table = ctx.autotune(jobs, repeats=1)
        assert len(table) == 18  # block 128 / 256 x tile 2 / 3 / 4 x unroll 1 / 16 / 64
        assert best in [t for t, _ in table]
        assert ctx.get_tuning() == best
        assert all(ms > 0 for _, ms in table)
    finally:
        ctx.close()


def test_batch_rejects_bad_jobs():
    ctx = mm3e_cuda.Context(0)
    try:
        s, cam = scenes.spheres_scene(32, 18)
        s.mode = abi.MODE_NORMAL
        cs = mm3e_cuda.CompiledScene(ctx, s)
        out = np.zeros((18, 32, 4), np.uint8)
        jobs = ctx.make_jobs([(cs, cam, 0, 0, abi.FB_RGBA8, None, out)])
        with pytest.raises(mm3e_cuda.RenderError) as ei:
            ctx.render_batch(jobs)
        assert ei.value.code == abi.ERR_UNSUPPORTED
        s2, _ = scenes.spheres_scene(32, 18)
        cs2 = mm3e_cuda.CompiledScene(ctx, s2)
        small = np.zeros((4, 4, 4), np.uint8)
        jobs = ctx.make_jobs([(cs2, cam, 0, 0, abi.FB_RGBA8, None, small)])
        jobs[0].out_bytes = small.nbytes
        with pytest.raises(mm3e_cuda.RenderError) as ei:
            ctx.render_batch(jobs)
        assert ei.value.code == abi.ERR_INVALID
    finally:
        ctx.close()
