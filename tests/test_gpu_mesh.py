"""GPU mesh -> SDF bake (mm3e_bake_mesh_sdf) against the oracle's restatement of bake_sdf.

Integer / index work (the BVH walk order, crossing parity) and binary32 arithmetic without
contraction on both sides: the baked samples must be bit-identical to the oracle's.
"""
import json

import numpy as np
import pytest

import mm3e_cuda
import oracle_py
from mm3e_cuda import abi, scenes
from parity import image_metrics

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["uv_sphere_28", "icosphere5_64", "icosphere5_128"])
def test_mesh_bake_bit_exact(gpu_ctx, case):
    if case == "uv_sphere_28":
        pos, tri = scenes.uv_sphere_mesh(12, 18, 1.0)
        res, pad = 28, 0.25
    else:
        pos, tri = scenes.displaced_icosphere(11, 5)
        res, pad = int(case.split("_")[1]), 0.1
    vol = gpu_ctx.bake_mesh_sdf(pos, tri, res, pad)
    dims, vmin, cell, ref = oracle_py.bake_mesh_sdf(pos, tri, res, pad)
    assert vol.dims == dims
    assert np.array_equal(np.asarray(vol.min, np.float32), vmin)
    assert np.array_equal(np.asarray(vol.cell, np.float32), cell)
    got = vol.data.reshape(ref.shape)
    diff = got != ref
    print(case, json.dumps({"dims": dims, "samples": int(ref.size), "differ": int(diff.sum()),
                            "inside": int((ref < 0).sum())}))
    assert not diff.any(), f"{int(diff.sum())} of {ref.size} samples differ"


def test_mesh_bake_device_output_and_errors(gpu_ctx):
    torch = pytest.importorskip("torch")
    pos, tri = scenes.uv_sphere_mesh(8, 12, 0.9)
    host = gpu_ctx.bake_mesh_sdf(pos, tri, 20, 0.2)
    n = host.data.size
    d = torch.zeros(n, dtype=torch.float32, device="cuda")
    dims, _, _ = gpu_ctx.bake_mesh_sdf(pos, tri, 20, 0.2, device_out=d.data_ptr())
    assert dims == host.dims
    assert np.array_equal(d.cpu().numpy(), host.data)
    with pytest.raises(mm3e_cuda.RenderError, match="padding must be positive and finite"):
        gpu_ctx.bake_mesh_sdf(pos, tri, 20, -1.0)
    flat = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0]], np.float32)
    with pytest.raises(mm3e_cuda.RenderError, match="no non-degenerate triangles"):
        gpu_ctx.bake_mesh_sdf(flat, np.array([[0, 1, 2]], np.uint32), 16, 0.1)


def test_mesh_volume_scene_render_parity(gpu_ctx):
    pos, tri = scenes.displaced_icosphere(5, 4)
    vol = gpu_ctx.bake_mesh_sdf(pos, tri, 48, 0.1)
    scene, cam = scenes.mesh_volume_scene(vol, seed=5, width=160, height=120)
    compiled = mm3e_cuda.CompiledScene(gpu_ctx, scene)
    gpu = compiled.render(cam, fmt=abi.FB_RGBA8)
    ref = mm3e_cuda.to_rgba8(oracle_py.render(scene.desc(), cam))
    m = image_metrics(gpu, ref)
    print("mesh_volume_scene", json.dumps(m))
    assert m["psnr"] >= 50.0 and m["within1_px"] >= 0.999, m
