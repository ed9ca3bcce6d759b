"""render_gbuffer / reprojection on the oracle, against the reference's engine tests
(mm3e-orchestrator/tests/engine.rs:185-255)."""
import numpy as np

import oracle_py
from mm3e_cuda import scenes
from mm3e_cuda.scene import orbit_camera, radians


def test_identity_reprojection_mostly_matches():
    s, c = scenes.demo_scene()
    g = oracle_py.render_gbuffer(s.desc(), c)
    out = oracle_py.reproject(g, c, c)
    same = (np.abs(out[..., 0].astype(int) - g["color"][..., 0].astype(int)) < 24).mean()
    assert same > 0.85


def test_hybrid_beats_the_cheap_fill():
    s, _ = scenes.demo_scene()
    c0 = orbit_camera((0.0, 0.8, 0.3), 7.0, 0.5, 0.3, radians(52.0))
    c1 = orbit_camera((0.0, 0.8, 0.3), 7.0, 0.62, 0.3, radians(52.0))
    g = oracle_py.render_gbuffer(s.desc(), c0)
    truth = oracle_py.render_gbuffer(s.desc(), c1)["color"]
    basic = oracle_py.reproject(g, c0, c1)
    hybrid = oracle_py.reproject(g, c0, c1, hybrid_handle=s.desc())
    err = lambda a: int(np.abs(a[..., 0].astype(int) - truth[..., 0].astype(int)).sum())
    assert err(hybrid) <= err(basic)


def test_object_motion_has_effect():
    s, c = scenes.demo_scene()
    g = oracle_py.render_gbuffer(s.desc(), c, movers=[(-1.2, 1.0, 0.0, 1.3)])
    assert (g["obj"] == 0).any()
    still = oracle_py.reproject(g, c, c, deltas=[(0.0, 0.0, 0.0)])
    moved = oracle_py.reproject(g, c, c, deltas=[(1.5, 0.0, 0.0)])
    assert not np.array_equal(still, moved)
