"""mm3e_march_rays_noalloc: ray queries that allocate no device memory.

It exists for callers that cannot allocate while they query (a frame loop casting picking or
collision rays cannot afford the device synchronisation of cudaMalloc/cudaFree; a service whose
memory is reserved up front has nothing left to allocate). Its results must equal those of the
allocating entry point mm3e_march_rays on the same rays, bit for bit (the march does not depend
on the launch), call after call, although every call reuses the same fixed scratch array; and a
call must leave the device's free memory as it was. The file is named so that pytest collects it
last.
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


class _DeviceBuffers:
    """Device inputs and outputs for up to n rays, allocated once (by torch) before the calls."""

    def __init__(self, n):
        self.torch = pytest.importorskip("torch")
        t = self.torch
        self.rays = t.zeros(6 * n, dtype=t.float32, device="cuda")
        self.t = t.empty(n, dtype=t.float32, device="cuda")
        self.m = t.empty(n, dtype=t.int32, device="cuda")
        self.s = t.empty(n, dtype=t.int32, device="cuda")

    def call(self, compiled, rays):
        n = len(rays)
        self.rays[:6 * n].copy_(self.torch.from_numpy(rays.reshape(-1)))
        self.torch.cuda.synchronize()  # the rays are complete before the call (it runs on its own stream)
        rc = lib().mm3e_march_rays_noalloc(compiled._ptr, C.c_void_p(self.rays.data_ptr()), n,
                                           C.c_void_p(self.t.data_ptr()), C.c_void_p(self.m.data_ptr()),
                                           C.c_void_p(self.s.data_ptr()))
        compiled.ctx.check(rc)
        return (self.t[:n].cpu().numpy(), self.m[:n].cpu().numpy().view(np.uint32),
                self.s[:n].cpu().numpy().view(np.uint32))


def test_noalloc_matches_allocating_entry_two_calls():
    ctx = mm3e_cuda.Context(0)
    try:
        scene, cam = scenes.gallery_scene(64, 36)
        compiled = mm3e_cuda.CompiledScene(ctx, scene)
        bufs = _DeviceBuffers(50000)
        for call, (n, seed) in enumerate(((50000, 1), (20000, 2))):
            rays = _rays(cam, n, seed)
            t_ref, m_ref, s_ref = compiled.march_rays(rays)
            t, m, s = bufs.call(compiled, rays)
            assert np.array_equal(m, m_ref), f"call {call}: material ids differ"
            assert np.array_equal(s, s_ref), f"call {call}: step counts differ"
            assert np.array_equal(t.view(np.uint32), t_ref.view(np.uint32)), f"call {call}: hit distances differ"
            assert (m != 0xFFFFFFFF).sum() > n // 4
    finally:
        ctx.close()


def test_noalloc_calls_leave_free_device_memory_unchanged():
    """After the first call (which may load the library's module and look up the array's
    address), calls of different sizes leave the device's free memory exactly as it was."""
    ctx = mm3e_cuda.Context(0)
    try:
        scene, cam = scenes.spheres_scene(64, 36)
        compiled = mm3e_cuda.CompiledScene(ctx, scene)
        bufs = _DeviceBuffers(200000)
        torch = bufs.torch
        bufs.call(compiled, _rays(cam, 1000, 3))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for n, seed in ((200000, 4), (7, 5), (65536, 6), (1, 7)):
            t, m, _ = bufs.call(compiled, _rays(cam, n, seed))
            assert len(t) == n
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
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
