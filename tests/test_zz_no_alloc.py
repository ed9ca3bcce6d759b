"""mm3e_march_rays_noalloc: ray queries that allocate no device memory.

It exists for callers that cannot allocate while they query (a frame loop casting picking or
collision rays cannot afford the device synchronisation of cudaMalloc/cudaFree; a service whose
memory is reserved up front has nothing left to allocate). Its results must equal those of the
allocating entry point mm3e_march_rays on the same rays, call after call, although every call
reuses the same fixed scratch array. The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import mm3e_cuda
from mm3e_cuda import abi, scenes
from mm3e_cuda.native import lib

pytestmark = pytest.mark.gpu


def _rays(cam, n, seed):
    rng = np.random.default_rng(seed)
    org = np.tile(np.array(cam.eye, np.float32), (n, 1))
    d = rng.normal(size=(n, 3)) * [0.35, 0.2, 0.35] + np.array(cam.forward)
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return np.ascontiguousarray(np.concatenate([org, d], axis=1), dtype=np.float32)


def _noalloc(compiled, rays):
    torch = pytest.importorskip("torch")
    n = len(rays)
    d_rays = torch.from_numpy(rays.reshape(-1)).cuda()
    d_t = torch.empty(n, dtype=torch.float32, device="cuda")
    d_m = torch.empty(n, dtype=torch.int32, device="cuda")
    d_s = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib().mm3e_march_rays_noalloc(compiled._ptr, C.c_void_p(d_rays.data_ptr()), n, C.c_void_p(d_t.data_ptr()),
                                       C.c_void_p(d_m.data_ptr()), C.c_void_p(d_s.data_ptr()))
    compiled.ctx.check(rc)
    return d_t.cpu().numpy(), d_m.cpu().numpy().view(np.uint32), d_s.cpu().numpy().view(np.uint32)


def test_noalloc_matches_allocating_entry_two_calls():
    ctx = mm3e_cuda.Context(0)
    try:
        scene, cam = scenes.gallery_scene(64, 36)
        compiled = mm3e_cuda.CompiledScene(ctx, scene)
        for call, (n, seed) in enumerate(((50000, 1), (20000, 2))):
            rays = _rays(cam, n, seed)
            t_ref, m_ref, s_ref = compiled.march_rays(rays)
            t, m, s = _noalloc(compiled, rays)
            assert np.array_equal(m, m_ref), f"call {call}: material ids differ"
            assert np.array_equal(s, s_ref), f"call {call}: step counts differ"
            assert np.allclose(t, t_ref, rtol=1e-6, atol=0.0), f"call {call}: hit distances differ"
            assert (m != 0xFFFFFFFF).sum() > n // 4
    finally:
        ctx.close()


def test_noalloc_rejects_oversized_batch():
    torch = pytest.importorskip("torch")
    ctx = mm3e_cuda.Context(0)
    try:
        scene, _ = scenes.spheres_scene(32, 18)
        compiled = mm3e_cuda.CompiledScene(ctx, scene)
        n = 262144 + 1
        buf = torch.zeros(6 * n, dtype=torch.float32, device="cuda")
        out = torch.zeros(n, dtype=torch.float32, device="cuda")
        rc = lib().mm3e_march_rays_noalloc(compiled._ptr, C.c_void_p(buf.data_ptr()), n, C.c_void_p(out.data_ptr()),
                                           C.c_void_p(out.data_ptr()), None)
        assert rc == abi.ERR_INVALID
        assert "262144" in lib().mm3e_last_error(ctx.handle).decode()
    finally:
        ctx.close()
