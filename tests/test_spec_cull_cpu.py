"""The specialised field's cull pre-tests never cull a member that the exact bound test keeps.

A LINEAR union member is skipped when its bound lower = |p - c| - r exceeds the best distance so
far (accel.rs:98-100). The generated code first tests squared distances with a relative margin
(far_beyond in device_math.cuh) for single members and for spatial clusters of members, skipping
the square root. These tests replay that arithmetic in IEEE binary32 (numpy float32: correctly
rounded, no contraction, as the device code compiled with --fmad=false; the generated pre-tests'
squared norms with their explicit fused multiply-adds, length_sq_fma) on adversarial points just
outside the cull boundary, and check the clusters' enclosing spheres in exact arithmetic.
"""
import re
from fractions import Fraction

import numpy as np

import mm3e_cuda
from mm3e_cuda import scenes

F = np.float32
M = F(1.00006103515625)  # 1 + 2^-14


def far_beyond(d2, bd, r):
    q = F(bd + r)
    return (bd >= F(0)) & (d2 > F(F(q * q) * M))


def length_sq(e):
    return F(F(F(e[..., 0] * e[..., 0]) + F(e[..., 1] * e[..., 1])) + F(e[..., 2] * e[..., 2]))


def fma32(a, b, c):
    """fl(a b + c) for float32 operands: the product is exact in binary64, the sum rounds there
    and then to binary32 (a double rounding that can differ from one fused rounding by one unit
    in rare ties, far inside the margins tested here)."""
    return F(np.float64(a) * np.float64(b) + np.float64(c))


def length_sq_fma(e):
    """device_math.cuh length_sq_fma: the squared norm the generated cull pre-tests take."""
    z2 = F(e[..., 2] * e[..., 2])
    return fma32(e[..., 0], e[..., 0], fma32(e[..., 1], e[..., 1], z2))


def _round32(x):
    """The binary32 value nearest the rational x (ties to even)."""
    f = np.float32(float(x))
    best = f
    for cand in (np.nextafter(f, F(-np.inf)), np.nextafter(f, F(np.inf))):
        dc, db = abs(Fraction(float(cand)) - x), abs(Fraction(float(best)) - x)
        if dc < db or (dc == db and (int(cand.view(np.uint32)) & 1) == 0):
            best = cand
    return best


def _fma(a, b, c):
    return _round32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


MU = F(1.0 - 2.0 ** -19)


def _lin_constants(c, r):
    """spec_gen.cpp lin_test's constants: -2c, mu |c|^2 rounded down, 2 M r and M r^2 rounded up."""
    M = Fraction(1) + Fraction(1, 2 ** 14)
    cc = sum(Fraction(float(x)) ** 2 for x in c) * Fraction(float(MU))
    c2 = np.float32(float(cc))
    if Fraction(float(c2)) > cc:
        c2 = np.nextafter(c2, F(-np.inf))
    up = lambda x: (lambda f: f if Fraction(float(f)) >= x else np.nextafter(f, F(np.inf)))(np.float32(float(x)))
    return (-2 * c).astype(F), c2, up(2 * M * Fraction(float(r))), up(M * Fraction(float(r)) ** 2)


def dist2_below_exact(p, c, base=None):
    """device_math.cuh dist2_below(p, cull_base(p), -2c, c2), every rounding exact."""
    a, c2, _, _ = _lin_constants(c, F(0))
    P2 = _fma(p[0], p[0], _fma(p[1], p[1], _round32(Fraction(float(p[2])) ** 2)))
    base = _round32(Fraction(float(P2)) * Fraction(float(MU)))
    s = _round32(Fraction(float(base)) + Fraction(float(c2)))
    return _fma(p[0], a[0], _fma(p[1], a[1], _fma(p[2], a[2], s)))


def far_beyond_lin_exact(p, c, r, bd):
    _, _, m2r, mr2 = _lin_constants(c, r)
    q = _fma(bd, _fma(bd, F(1.00006103515625), m2r), mr2)
    return bool(bd >= 0) and dist2_below_exact(p, c) > q


def exact_lower(p, c, r):
    e = (p - c).astype(F)
    return F(np.sqrt(length_sq(e)).astype(F) - r)


def _points_near(rng, c, radius, n):
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    scale = radius * (1.0 + rng.uniform(-2e-4, 2e-4, n))
    return (c.astype(np.float64) + d * scale[:, None]).astype(F)


def test_member_pretest_implies_exact_cull():
    rng = np.random.default_rng(11)
    for _ in range(40):
        c = rng.uniform(-50, 50, 3).astype(F)
        r = F(rng.choice([0.0, rng.uniform(1e-3, 8.0)]))
        bd = F(rng.choice([0.0, rng.uniform(1e-6, 1e-2), rng.uniform(0.01, 30.0)]))
        p = _points_near(rng, c, float(bd) + float(r), 20000)
        lower = exact_lower(p, c, r)
        culled = lower > bd
        for norm in (length_sq, length_sq_fma):  # the interpreter's pre-test and the generated one
            d2 = norm((p - c).astype(F))
            skip = far_beyond(d2, bd, r)
            assert (lower[skip] > bd).all()
            # the margin is narrow: most points the exact test culls are culled by the pre-test too
            if culled.sum() > 1000:
                assert skip.sum() >= 0.5 * culled.sum()


def test_negative_best_is_never_pretested():
    d2 = np.array([1e6], F)
    assert not far_beyond(d2, F(-0.5), F(1.0)).any()


def _clusters(src):
    """(centre, radius, [(member centre, member radius)]) of every cluster in generated source: a
    cluster's centre is -1/2 of its linearised test's -2c constants, its radius is in the line's
    comment; a member's centre and radius are in its bound distance line (length(p - c) - r)."""
    hexf = lambda h: np.array([int(h, 16)], np.uint32).view(F)[0]
    H = r"__uint_as_float\(0x(\w+)u\)"
    out, cur = [], None
    for line in src.splitlines():
        m = re.search(r"far_beyond_lin\(dist2_below\(p, CB, " + H + ", " + H + ", " + H + ", " + H +
                      r"\), bd, " + H + ", " + H + r"\)\) \{  // cluster of \d+, radius " + H, line)
        if m:
            c = np.array([hexf(m.group(i)) for i in (1, 2, 3)], F) * F(-0.5)
            cur = (c.astype(F), hexf(m.group(7)), [])
            out.append(cur)
            continue
        m = re.search(r"const float lower = length\(p - V\{" + H + ", " + H + ", " + H + r"\}\) - " + H + ";", line)
        if m and cur is not None:
            cur[2].append((np.array([hexf(m.group(i)) for i in (1, 2, 3)], F), hexf(m.group(4))))
        if "// end of cluster" in line:
            cur = None
    return out


def _exact_norm_le(v, bound):
    """|v| <= bound in exact rational arithmetic (v, bound: float32 values)."""
    s = sum(Fraction(float(x)) ** 2 for x in v)
    b = Fraction(float(bound))
    return b >= 0 and s <= b * b


def test_cluster_spheres_enclose_members_and_cull_safely():
    rng = np.random.default_rng(5)
    sources = [mm3e_cuda.spec_source(scenes.gallery_scene(64, 36)[0]),
               mm3e_cuda.spec_source(scenes.procedural_scene(3, 64, 48)[0]),
               mm3e_cuda.spec_source(scenes.canonical_asset_scene()[0])]
    n_clusters = 0
    for src in sources:
        for C, R, members in _clusters(src):
            assert len(members) >= 2
            n_clusters += 1
            for c, r in members:
                # |C - c| + r <= R exactly
                assert _exact_norm_le((C.astype(np.float64) - c.astype(np.float64)), Fraction(float(R)) - Fraction(float(r)))
            for bd in (F(0.0), F(1e-4), F(0.3), F(4.0)):
                p = _points_near(rng, C, float(bd) + float(R), 20000)
                skip = far_beyond(length_sq_fma((p - C).astype(F)), bd, R)
                for c, r in members:
                    assert (exact_lower(p[skip], c, r) > bd).all()
                # the linearised test the generated code takes
                pts = p[rng.choice(len(p), 150, replace=False)]
                skip = np.array([far_beyond_lin_exact(q, C, R, bd) for q in pts])
                for c, r in members:
                    assert (exact_lower(pts[skip], c, r) > bd).all()
    assert n_clusters >= 2


def _zero_with_sign_and(a, b):
    bits = (a.view(np.uint32) & b.view(np.uint32)) & np.uint32(0x80000000)
    return bits.view(np.float32)


def test_identity_rotation_shortcut_is_bit_exact():
    """An object whose rotation is exactly the identity skips the rotation's multiplications
    (rot_t_identity in device_math.cuh): x = vx + (a zero with the sign of vy AND vz), and so on.
    Checked bit for bit against the full product r[0]·vx + r[1]·vy + r[2]·vz of the identity in
    binary32 (vec.rs:125-127 order) on signed zeros, subnormals and ordinary values."""
    F = np.float32
    special = np.array([0.0, -0.0, 1e-45, -1e-45, 1.5e-39, -2.5e-39, 1.0, -1.0, 3.25, -7.5e3, 6e37, -6e37], F)
    rng = np.random.default_rng(5)
    rand = (rng.standard_normal(4000) * 10.0 ** rng.integers(-6, 6, 4000)).astype(F)
    vals = np.concatenate([special, rand])
    g = np.array(np.meshgrid(special, special, special, indexing="ij")).reshape(3, -1)
    v = np.concatenate([g, rng.choice(vals, (3, 20000))], axis=1).astype(F)
    vx, vy, vz = v
    one, zero = F(1.0), F(0.0)
    full = [(one * vx + zero * vy) + zero * vz, (zero * vx + one * vy) + zero * vz, (zero * vx + zero * vy) + one * vz]
    short = [vx + _zero_with_sign_and(vy, vz), vy + _zero_with_sign_and(vx, vz), vz + _zero_with_sign_and(vx, vy)]
    for f, s in zip(full, short):
        assert f.dtype == s.dtype == np.float32
        assert np.array_equal(f.view(np.uint32), s.view(np.uint32))
    # the generator drops the rotation from an identity member's weak-bound test and the RO table
    scene, _ = scenes.gallery_scene(32, 18)
    src = mm3e_cuda.spec_source(scene)
    assert "weak_beyond_sq(scale(p - V{" in src


def _smooth_union_d(a, b, k):
    """sdf.rs:152-160 distance in binary32 (a, b arrays, k > 0)."""
    h = F(F(0.5) + F(F(F(0.5) * F(b - a)) / k))
    h = np.minimum(np.maximum(h, F(0)), F(1)).astype(F)
    one_h = F(F(1) - h)
    return F(F(F(b * one_h) + F(a * h)) - F(F(k * h) * one_h)), h


def test_far_one_segments_leave_the_accumulator():
    """A smooth-union segment is skipped where its sphere distance clears max(acc + k rounded up,
    slack) by the squared pre-test (acc finite and non-zero): there the blend weight is exactly 1, and
    the blend returns the accumulator's distance bit for bit with its material. A union segment
    (threshold acc) keeps the accumulator outright, a subtraction (threshold -acc) keeps it as
    max(acc, -lower). Both the specialised field and the interpreter (one_keeps_acc) apply it."""
    rng = np.random.default_rng(23)
    slack = F(0.4)
    for _ in range(60):
        c = rng.uniform(-20, 20, 3).astype(F)
        r = F(rng.uniform(0.05, 3.0))
        k = F(rng.choice([0.01, 0.3, 1.0, 2.5]))
        acc = np.concatenate([rng.uniform(-5, 5, 8000), rng.uniform(-150, 150, 6000),
                              rng.uniform(1e-6, 1e-3, 6000)]).astype(F)
        acc[acc == 0] = F(1e-3)
        exact = acc.astype(np.float64) + np.float64(k)  # exact: the operands' exponents are close
        up = exact.astype(F)
        up = np.where(up.astype(np.float64) < exact, np.nextafter(up, F(np.inf)), up).astype(F)  # __fadd_ru
        thr = np.maximum(up, slack).astype(F)
        p = _points_near(rng, c, float(rng.uniform(0.5, 40.0)), 20000)
        p = (c + (p - c) * rng.uniform(0.0, 3.0, (20000, 1))).astype(F)
        d2 = length_sq((p - c).astype(F))
        skip = far_beyond(d2, thr, r)
        lower = exact_lower(p, c, r)
        assert skip.mean() > 0.05
        assert (lower[skip] > slack).all()  # the slack substitute is the member's value there
        dist, h = _smooth_union_d(acc, lower, k)
        assert (h[skip] == F(1)).all()
        assert np.array_equal(dist[skip].view(np.uint32), acc[skip].view(np.uint32))
        # the union's skip (threshold max(acc, slack)) keeps the accumulator: acc <= lower
        uskip = far_beyond(d2, np.maximum(acc, slack).astype(F), r)
        assert (acc[uskip] <= lower[uskip]).all()
        # the subtraction's skip (threshold max(-acc, slack)): max(acc, -lower) is acc, bit for bit
        sskip = far_beyond(d2, np.maximum(-acc, slack).astype(F), r)
        assert sskip.mean() > 0.05
        sub = np.fmax(acc, -lower).astype(F)
        assert np.array_equal(sub[sskip].view(np.uint32), acc[sskip].view(np.uint32))


def test_smooth_skip_holds_for_large_accumulators_and_small_blends():
    """The smooth-union skip's threshold is acc + k rounded up, so it needs no bound on |acc|:
    sphere distances within a few parts in 10^4 of the threshold (the pre-test keeps a 2^-14
    margin on squared distances), accumulators up to 10^5, blend radii down to 10^-3."""
    rng = np.random.default_rng(31)
    slack = F(0.4)
    for k in (0.001, 0.01, 0.3, 2.0):
        k = F(k)
        acc = np.concatenate([rng.uniform(1e2, 1e5, 20000), rng.uniform(0.4, 3.0, 20000)]).astype(F)
        r = F(0.75)
        exact = acc.astype(np.float64) + np.float64(k)
        up = exact.astype(F)
        up = np.where(up.astype(np.float64) < exact, np.nextafter(up, F(np.inf)), up).astype(F)
        thr = np.maximum(up, slack).astype(F)
        dist_c = (thr.astype(np.float64) + np.float64(r)) * (1.0 + rng.uniform(-1e-4, 2e-4, len(acc)))
        d2 = F(dist_c * dist_c)
        skip = far_beyond(d2, thr, r)
        assert 0.2 < skip.mean() < 0.8
        lower = F(np.sqrt(d2).astype(F) - r)
        dist, h = _smooth_union_d(acc, lower, k)
        assert (h[skip] == F(1)).all()
        assert np.array_equal(dist[skip].view(np.uint32), acc[skip].view(np.uint32))


def test_axis_plane_is_the_plane_field_bit_for_bit():
    """An axis-aligned plane (+-1 on one axis, +0 on the others, identity rotation, offset other
    than -0) is generated as fl(+-l_k + h) with l_k = (p_k - pos_k) inv (spec_gen.cpp axis_plane).
    Checked bit for bit against the field the interpreter takes, dot(l, n) + h with l the
    identity-rotated, scaled local point (vec.rs:24-26 order; rot_t_identity), on signed zeros,
    subnormals and ordinary coordinates, for every axis, sign, offset and scale tested."""
    special = np.array([0.0, -0.0, 1e-45, -1e-45, 1.5e-39, -2.5e-39, 1.0, -1.0, 3.25, -7.5e3, 0.5, -0.25], F)
    g = np.stack(np.meshgrid(special, special, special, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(3)
    g = np.concatenate([g, rng.uniform(-20, 20, (4000, 3)).astype(F)])
    for k in range(3):
        for sign in (F(1.0), F(-1.0)):
            for h in (F(0.0), F(4.0), F(-2.5), F(1e-30)):
                for pos, inv in ((np.zeros(3, F), F(1.0)), (np.array([0.25, -1.5, 0.5], F), F(0.5))):
                    n = np.zeros(3, F)
                    n[k] = sign
                    d = (g - pos).astype(F)
                    r = np.stack([F(d[:, 0] + _zero_with_sign_and(d[:, 1], d[:, 2])),
                                  F(d[:, 1] + _zero_with_sign_and(d[:, 0], d[:, 2])),
                                  F(d[:, 2] + _zero_with_sign_and(d[:, 0], d[:, 1]))], -1)
                    l = (r * inv).astype(F)
                    ref = F(F(F(F(l[:, 0] * n[0]) + F(l[:, 1] * n[1])) + F(l[:, 2] * n[2])) + h)
                    lk = F(F(g[:, k] - pos[k]) * inv)
                    fast = F((lk if sign > 0 else -lk) + h)
                    assert np.array_equal(ref.view(np.uint32), fast.view(np.uint32)), (k, sign, h)


def test_linearised_distance_never_exceeds_the_squared_distance():
    """dist2_below (|p|^2 mu + mu |c|^2 - 2 p.c in fused multiply-adds) is a lower bound of
    |p - c|^2 in exact arithmetic: on points all over, near c (where the difference cancels) and
    far away, with every binary32 rounding done exactly."""
    rng = np.random.default_rng(2)
    for it in range(3000):
        c = (rng.standard_normal(3) * rng.uniform(0, 30)).astype(F)
        if it % 3 == 0:
            p = (c + rng.standard_normal(3) * 10.0 ** rng.uniform(-6, 0)).astype(F)
        else:
            p = (rng.standard_normal(3) * 10.0 ** rng.uniform(-2, 2.5)).astype(F)
        exact = sum((Fraction(float(p[i])) - Fraction(float(c[i]))) ** 2 for i in range(3))
        assert Fraction(float(dist2_below_exact(p, c))) <= exact, (p, c)


def test_linearised_pretest_implies_exact_cull():
    """far_beyond_lin never culls a member that the exact bound test keeps, on points just outside
    the cull boundary; 2% beyond it, it culls them all."""
    rng = np.random.default_rng(13)
    for _ in range(30):
        c = rng.uniform(-50, 50, 3).astype(F)
        r = F(rng.choice([0.0, rng.uniform(1e-3, 8.0)]))
        bd = F(rng.choice([0.0, rng.uniform(1e-6, 1e-2), rng.uniform(0.01, 30.0)]))
        p = _points_near(rng, c, float(bd) + float(r), 200)
        lower = exact_lower(p, c, r)
        skip = np.array([far_beyond_lin_exact(q, c, r, bd) for q in p])
        assert (lower[skip] > bd).all()
        if float(bd) + float(r) > 0.5:
            far = _points_near(rng, c, (float(bd) + float(r)) * 1.02, 50)
            assert all(far_beyond_lin_exact(q, c, r, bd) for q in far)
    assert not far_beyond_lin_exact(np.array([1e3, 0, 0], F), np.zeros(3, F), F(1.0), F(-0.5))


def test_enclosing_sphere_covers_every_test_inside():
    """The enclosing sphere over a union run's sphere tests (spec_gen.cpp enclosing_sphere) contains
    every cluster sphere and every member bound sphere inside its block, in exact arithmetic, so
    a sample beyond it would be culled by each of them."""
    hexf = lambda h: np.array([int(h, 16)], np.uint32).view(F)[0]
    H = r"__uint_as_float\(0x(\w+)u\)"
    n_super = 0
    for src in (mm3e_cuda.spec_source(scenes.gallery_scene(64, 36)[0]),):
        inside = None
        for line in src.splitlines():
            m = re.search(r"dist2_below\(p, CB, " + H + ", " + H + ", " + H + r".*// enclosing sphere of \d+ tests, radius " + H, line)
            if m:
                inside = (np.array([hexf(m.group(i)) for i in (1, 2, 3)], F) * F(-0.5), hexf(m.group(4)), [])
                n_super += 1
                continue
            if inside is None:
                continue
            m = re.search(r"dist2_below\(p, CB, " + H + ", " + H + ", " + H + r".*// cluster of \d+, radius " + H, line)
            if m:
                inside[2].append((np.array([hexf(m.group(i)) for i in (1, 2, 3)], F) * F(-0.5), hexf(m.group(4))))
            m = re.search(r"length\(p - V\{" + H + ", " + H + ", " + H + r"\}\) - " + H, line)
            if m:
                inside[2].append((np.array([hexf(m.group(i)) for i in (1, 2, 3)], F), hexf(m.group(4))))
            if "// end of enclosing sphere" in line:
                C, R, parts = inside
                assert len(parts) >= 3
                for c, r in parts:
                    assert _exact_norm_le(C.astype(np.float64) - c.astype(np.float64), Fraction(float(R)) - Fraction(float(r)))
                inside = None
    assert n_super >= 1
