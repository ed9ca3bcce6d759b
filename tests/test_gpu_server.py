"""Served form (mm3e_server): continuous batching, admission against an HBM budget.

The spec bar for serving: each result is the same alone and in the mix. Here a request
rendered alone (submitted and waited for on its own) and the same request inside a stream of
overlapping requests of other scenes and sizes give byte-identical frames, and both equal the
plain per-frame call on a separate context (itself checked against the CPU oracle).
"""
import numpy as np
import pytest

import mm3e_cuda
from mm3e_cuda import abi, scenes

pytestmark = pytest.mark.gpu


def _stream(seed, n):
    """A small mixed stream: camera updates of resident procedural scenes, new scenes, and one
    mesh-baked scene. Returns (resident scenes, [(kind, scene or index, camera, w, h)])."""
    rng = np.random.default_rng(seed)
    resident = [scenes.procedural_scene(100 + i, 64, 48) for i in range(3)]
    items = []
    for k in range(n):
        u = rng.random()
        w, h = [(64, 48), (40, 40), (96, 54), (33, 21)][int(rng.integers(0, 4))]
        if u < 0.6:
            i = int(rng.integers(0, len(resident)))
            s, _ = resident[i]
            cam = mm3e_cuda.scene.orbit_camera((0.0, 0.0, 0.0), float(rng.uniform(9, 14)),
                                               float(rng.uniform(-3, 3)), float(rng.uniform(0.1, 0.6)), 0.8)
            items.append(("resident", i, cam, w, h))
        elif u < 0.9:
            s, cam = scenes.procedural_scene(200 + k, w, h)
            items.append(("new", s, cam, w, h))
        else:
            items.append(("mesh", k, None, w, h))
    return resident, items


def _mesh_scene(k, w, h):
    pos, tri = scenes.displaced_icosphere(k % 3, 3)
    from mm3e_cuda.scene import SdfVolume
    placeholder = SdfVolume((2, 2, 2), (0, 0, 0), (1, 1, 1), np.zeros(8, np.float32))
    s, cam = scenes.mesh_volume_scene(placeholder, seed=k, width=w, height=h)
    s.marcher.normal_h = 0.02
    return s, cam, (pos, tri)


def _requests(srv, resident_ids, resident, items):
    reqs, keeps, outs = [], [], []
    for kind, what, cam, w, h in items:
        out = np.zeros((h, w, 4), np.uint8)
        if kind == "resident":
            r, keep = srv.request(cam, out, scene_id=resident_ids[what], width=w, height=h)
        elif kind == "new":
            r, keep = srv.request(cam, out, new_scene=what, width=w, height=h)
        else:
            s, cam, mesh = _mesh_scene(what, w, h)
            r, keep = srv.request(cam, out, new_scene=s, mesh=mesh, mesh_volume=0, mesh_resolution=40,
                                  mesh_padding=0.1, width=w, height=h)
        reqs.append(r)
        keeps.append(keep)
        outs.append(out)
    return reqs, keeps, outs


def _wait_specialized(srv, n, timeout_s=300.0):
    """Poll the server until its background compiles are done; returns its stats."""
    import time
    t0 = time.time()
    while True:
        st = srv.stats()
        if st["spec_pending"] == 0 and st["scenes_specialized"] >= n:
            return st
        assert time.time() - t0 < timeout_s, st
        time.sleep(0.05)


@pytest.mark.parametrize("mode", ["batched", "plain", "specialized"])
def test_alone_equals_in_mix(mode):
    """In the "specialized" mode the resident scenes' kernels are compiled in the background
    (spec_workers) and their requests render with them beside the coalesced pass sequences."""
    plain = mode == "plain"
    ctx = mm3e_cuda.Context(0)
    srv = mm3e_cuda.Server(ctx, max_inflight=2, plain=plain, spec_workers=4 if mode == "specialized" else 0)
    try:
        resident, items = _stream(7, 24)
        ids = [srv.add_scene(s) for s, _ in resident]
        if mode == "specialized":
            _wait_specialized(srv, len(resident))
        # alone: one request at a time
        reqs, keeps, alone = _requests(srv, ids, resident, items)
        for r in reqs:
            t = srv.submit(r)
            res = srv.wait(t)
            assert res["status"] == abi.OK
        # in the mix: all arrive within a few milliseconds, overlapping on the device
        reqs2, keeps2, mixed = _requests(srv, ids, resident, items)
        arrivals = [0.0005 * i for i in range(len(reqs2))]
        rc, res = srv.replay(reqs2, arrivals)
        assert rc == abi.OK, res
        for i, (a, b) in enumerate(zip(alone, mixed)):
            assert np.array_equal(a, b), f"request {i} ({items[i][0]}) differs alone vs in the mix"
        st = srv.stats()
        assert st["completed"] == 2 * len(items) and st["failed"] == 0
        if mode == "batched":
            assert st["frames_in_sequences"] > st["sequences"], st  # requests were coalesced
        if mode == "specialized":
            n_resident = sum(1 for it in items if it[0] == "resident")
            assert st["scenes_specialized"] == len(resident) and st["spec_frames"] == 2 * n_resident, st
        else:
            assert st["spec_frames"] == 0, st
        assert st["mesh_bakes"] >= 1 and st["mesh_bake_hits"] >= 1
    finally:
        srv.close()
        ctx.close()
    # cross-check against the plain per-frame call on a separate context
    ctx2 = mm3e_cuda.Context(0)
    try:
        for i, (kind, what, cam, w, h) in enumerate(items):
            if kind == "resident":
                s, _ = scenes.procedural_scene(100 + what, w, h)
            elif kind == "new":
                s = what
            else:
                continue
            ref = mm3e_cuda.CompiledScene(ctx2, s).render(cam, fmt=abi.FB_RGBA8)
            assert np.array_equal(ref, alone[i]), f"request {i} differs from the plain per-frame call"
    finally:
        ctx2.close()


def _sphere_volume(n, radius):
    from mm3e_cuda.scene import SdfVolume
    ax = np.linspace(-1.5, 1.5, n, dtype=np.float32)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    d = (np.sqrt(x * x + y * y + z * z) - radius).astype(np.float32)
    cell = float(ax[1] - ax[0])
    return SdfVolume((n, n, n), (-1.5, -1.5, -1.5), (cell, cell, cell), d)


def test_budget_waits_and_evicts_but_completes():
    ctx = mm3e_cuda.Context(0)
    kw = dict(max_samples=1 << 18, max_inflight=2)
    probe = mm3e_cuda.Server(ctx, **kw)
    reserved = probe.stats()["reserved_bytes"]
    probe.close()
    assert reserved > 0
    # room for the slot buffers plus about two 4 MB frames and a few 1 MB scene volumes
    srv = mm3e_cuda.Server(ctx, hbm_budget_bytes=reserved + (11 << 20), **kw)
    try:
        outs, tickets, keeps = [], [], []
        for k in range(8):
            s, cam = scenes.mesh_volume_scene(_sphere_volume(64, 0.6 + 0.05 * k), seed=k, width=512, height=512)
            out = np.zeros((512, 512, 4), np.float32)
            r, keep = srv.request(cam, out, new_scene=s, fmt=abi.FB_RGBA_F32)
            tickets.append(srv.submit(r))
            keeps.append((r, keep))
            outs.append((out, s, cam))
        for t in tickets:
            assert srv.wait(t)["status"] == abi.OK
        st = srv.stats()
        assert st["peak_admitted_bytes"] + st["reserved_bytes"] <= st["budget_bytes"], st
        assert st["scenes_evicted"] >= 1, st
        # a frame that can never fit is refused with the budget error
        big = np.zeros((4096, 4096, 4), np.float32)
        s, cam = scenes.procedural_scene(999, 64, 64)
        r, keep = srv.request(cam, big, new_scene=s, width=4096, height=4096, fmt=abi.FB_RGBA_F32)
        assert srv.wait(srv.submit(r))["status"] == abi.ERR_BUDGET
    finally:
        srv.close()
        ctx.close()
    ctx2 = mm3e_cuda.Context(0)
    try:
        for out, s, cam in outs[:3]:
            assert np.array_equal(out, mm3e_cuda.CompiledScene(ctx2, s).render(cam, fmt=abi.FB_RGBA_F32))
    finally:
        ctx2.close()


def test_unknown_scene_and_bad_requests_fail_cleanly():
    ctx = mm3e_cuda.Context(0)
    srv = mm3e_cuda.Server(ctx)
    try:
        s, cam = scenes.spheres_scene(32, 18)
        out = np.zeros((18, 32, 4), np.uint8)
        r, keep = srv.request(cam, out, scene_id=12345)
        t = srv.submit(r)
        assert srv.wait(t)["status"] == abi.ERR_INVALID
        sid = srv.add_scene(s)
        r, keep = srv.request(cam, out, scene_id=sid)
        assert srv.wait(srv.submit(r))["status"] == abi.OK
        s.mode = abi.MODE_NORMAL
        with pytest.raises(mm3e_cuda.RenderError):
            srv.add_scene(s)
    finally:
        srv.close()
        ctx.close()
