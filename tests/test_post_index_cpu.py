"""Index arithmetic of the fused bloom kernels (k_bloom_h / k_bloom_v in post_kernels.cuh), replayed
on the CPU: blur4's four outputs read each tap once, and every output still sums the reference's
taps (post.rs:348-368) in kernel order with the right weights; every shared-memory window read
of the horizontal pass stays inside the window, whatever the job layout, radius or row width."""
import random

SEG, HALO = 256 * 4, 32
WIN = SEG + 2 * HALO


def _clamp(v, lo, hi):
    return min(max(v, lo), hi)


def _blur4(r, tap):
    """(tap index, weight index) sequence of each of blur4's outputs, in summation order."""
    seq = [[], [], [], []]

    def add(o, j, k):
        seq[o].append((tap(j), k))

    add(0, 0, 0)
    add(0, 1, 1)
    add(1, 1, 0)
    add(0, 2, 2)
    add(1, 2, 1)
    add(2, 2, 0)
    c1, c2, c3 = 2, 1, 0
    for j in range(3, 2 * r + 1):
        add(0, j, j)
        add(1, j, c1)
        add(2, j, c2)
        add(3, j, c3)
        c3, c2, c1 = c2, c1, j
    add(1, 2 * r + 1, c1)
    add(2, 2 * r + 1, c2)
    add(3, 2 * r + 1, c3)
    add(2, 2 * r + 2, c1)
    add(3, 2 * r + 2, c2)
    add(3, 2 * r + 3, c1)
    return seq


def test_horizontal_windows_and_tap_order():
    rnd = random.Random(1)
    checked = 0
    for _ in range(60):
        jobs, base = [], 0
        for _ in range(rnd.randint(1, 4)):
            w, h = rnd.choice([1, 2, 3, 5, 7, 13, 64, 70, 255, 1024, 1921]), rnd.choice([1, 2, 3, 7])
            jobs.append((base, w, h, rnd.choice([1, 2, 3, 12, 31, 32]), rnd.random() < 0.8))
            base += w * h
        n = base

        def job_of(i):
            return next(j for j in jobs if j[0] <= i < j[0] + j[1] * j[2])

        for seg in range(0, n, SEG):
            lo = seg - HALO
            for t in range(256):
                i0 = seg + 4 * t
                if i0 >= n:
                    continue
                pb, w, h, r, bloom = job_of(i0)
                x0, y = (i0 - pb) % w, (i0 - pb) // w
                if not (bloom and x0 + 3 < w and 1 <= r <= HALO):
                    continue  # the per-pixel path, which checks its window bounds itself
                row_e = pb + y * w - lo

                def tap(j):
                    e = row_e + _clamp(x0 - r + j, 0, w - 1)
                    assert 0 <= e < WIN
                    return e + lo

                seq = _blur4(r, tap)
                for o in range(4):
                    want = [(pb + y * w + _clamp(x0 + o + ki - r, 0, w - 1), ki) for ki in range(2 * r + 1)]
                    assert seq[o] == want
                    checked += 1
    assert checked > 10000


def test_vertical_groups_and_tap_order():
    rnd = random.Random(2)
    for _ in range(80):
        w, h, r = rnd.randint(1, 24), rnd.randint(1, 24), rnd.randint(1, 40)
        for g in range(w * ((h + 3) // 4)):
            x, y0 = g % w, (g // w) * 4
            seq = _blur4(r, lambda j: _clamp(y0 - r + j, 0, h - 1) * w + x)
            for o in range(4):
                if y0 + o < h:
                    assert seq[o] == [(_clamp(y0 + o + ki - r, 0, h - 1) * w + x, ki) for ki in range(2 * r + 1)]


def test_window_swizzle_is_a_conflict_free_permutation():
    """win_slot(e) = e ^ ((e >> 3) & 3): a permutation of each run of eight 16-byte slots under
    which the eight lanes of a quarter warp reading elements four apart hit eight different bank
    groups, and so do eight consecutive elements (the window fill)."""
    def slot(e):
        return e ^ ((e >> 3) & 3)

    assert sorted(slot(e) for e in range(WIN)) == list(range(WIN))
    for base in range(0, WIN - 128):
        for q in range(4):
            assert len({slot(base + 4 * (8 * q + t)) % 8 for t in range(8)}) == 8
    for start in range(0, WIN, 8):
        assert len({slot(e) % 8 for e in range(start, start + 8)}) == 8
