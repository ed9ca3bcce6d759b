"""Mesh -> SDF bake: the oracle against the reference's own known answers, and the mesh
generators of the served stream (CPU only)."""
from collections import Counter

import numpy as np
import pytest

import oracle_py
from mm3e_cuda import scenes
from mm3e_cuda.scene import Object, Prim, Scene, Transform, Material


def test_x_crossing_shared_diagonal_counted_once():
    # mm3e-kit/src/triangle.rs:43-54
    a, b, c, d = (2.0, -1.0, -1.0), (2.0, 1.0, -1.0), (2.0, 1.0, 1.0), (2.0, -1.0, 1.0)
    for tris in ([[a, b, c], [a, c, d]], [[c, b, a], [d, c, a]], [[a, c, b], [a, c, d]]):
        for y in (-0.7, 0.0, 0.4, 0.75):
            hits = [x for x in (oracle_py.x_crossing(t[0], t[1], t[2], y, y) for t in tris) if x is not None]
            assert hits == [2.0]


def test_x_crossing_projected_vertices_and_thin_faces():
    # mm3e-kit/src/triangle.rs:56-67
    o = (1.0, 0.0, 0.0)
    p = [(1.0, -1.0, -1.0), (1.0, 1.0, -1.0), (1.0, 1.0, 1.0), (1.0, -1.0, 1.0)]
    hits = sum(oracle_py.x_crossing(o, p[i], p[(i + 1) % 4], 0.0, 0.0) is not None for i in range(4))
    assert hits == 1
    assert oracle_py.x_crossing(o, (1.0, 1e-7, 0.0), (1.0, 0.0, 1e-7), 2e-8, 2e-8) == 1.0


def _volume_field(dims, vmin, cell, data, pts):
    from mm3e_cuda.scene import SdfVolume
    s = Scene(8, 8)
    m = s.material(Material.solid((0.5, 0.5, 0.5)))
    vid = s.volume(SdfVolume(dims, vmin, cell, data))
    s.add(Object(Prim.volume(vid), Transform.IDENTITY, m))
    d, _ = oracle_py.field(s.desc(), np.asarray(pts, np.float32))
    return d


def test_bake_sphere_known_answer():
    # mm3e-orchestrator/tests/engine.rs:403-420: uv sphere (12, 18, 1.0), resolution 28, padding 0.25
    pos, tri = scenes.uv_sphere_mesh(12, 18, 1.0)
    dims, vmin, cell, data = oracle_py.bake_mesh_sdf(pos, tri, 28, 0.25)
    pts = [(0.0, 0.0, 0.0), (1.2, 0.0, 0.0), (0.0, 1.2, 0.0)]
    got = _volume_field(dims, vmin, cell, data, pts)
    for p, g in zip(pts, got):
        want = np.linalg.norm(p) - 1.0
        assert abs(g - want) < 0.16, (p, g, want)
    assert data.min() < 0 < data.max()


def test_bake_errors_match_reference_messages():
    pos, tri = scenes.uv_sphere_mesh(6, 8, 1.0)
    with pytest.raises(ValueError, match="padding must be positive and finite"):
        oracle_py.bake_mesh_sdf(pos, tri, 16, 0.0)
    with pytest.raises(ValueError, match="references a vertex out of range"):
        oracle_py.bake_mesh_sdf(pos, np.array([[0, 1, 10_000]], np.uint32), 16, 0.1)
    bad = pos.copy()
    bad[3, 1] = np.nan
    with pytest.raises(ValueError, match="mesh vertex 3 is non-finite"):
        oracle_py.bake_mesh_sdf(bad, tri, 16, 0.1)
    flat = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0]], np.float32)
    with pytest.raises(ValueError, match="no non-degenerate triangles"):
        oracle_py.bake_mesh_sdf(flat, np.array([[0, 1, 2]], np.uint32), 16, 0.1)


def test_bake_grid_dims_follow_longest_axis():
    pos = np.array([[0, 0, 0], [2, 0, 0], [0, 1, 0], [0, 0, 0.5]], np.float32)
    tri = np.array([[0, 1, 2], [0, 2, 3], [0, 3, 1], [1, 3, 2]], np.uint32)
    dims, vmin, cell, _ = oracle_py.bake_mesh_sdf(pos, tri, 21, 0.5, grid_only=True)
    # padded size (3, 2, 1.5): longest axis gets the resolution, others round((s/3)*20)+1
    assert dims == (21, 14, 11)
    assert np.allclose(vmin, [-0.5, -0.5, -0.5])


def test_icosphere_generator_is_closed_and_sized():
    v, f = scenes.icosphere(3)
    assert len(v) == 10 * 4 ** 3 + 2 and len(f) == 20 * 4 ** 3
    edges = Counter()
    for a, b, c in f:
        for x, y in ((a, b), (b, c), (c, a)):
            edges[(min(x, y), max(x, y))] += 1
    assert set(edges.values()) == {2}
    pos, tri = scenes.displaced_icosphere(7, 5)
    assert len(tri) == 20480 and len(pos) == 10242
    r = np.linalg.norm(pos, axis=1)
    assert 0.8 < r.min() and r.max() < 1.2
    again, _ = scenes.displaced_icosphere(7, 5)
    assert np.array_equal(pos, again)
    other, _ = scenes.displaced_icosphere(8, 5)
    assert not np.array_equal(pos, other)
