"""The empty-box crossing of the traversal kernels (vt_device.cuh: cross_region, prefix_count,
finish_axis, advance_axis), restated in binary32 with numpy and checked against iterating the
DDA step it replaces (trace.frag:83-86: every axis whose side distance equals the minimum adds its
delta and moves one voxel) until some axis takes its last move to the box face.

Final side distances, moves per axis and the axes stepped on the last iteration must be identical.
The cases are random boxes and side distances, ties (equal sides and deltas), axes that do not step
(side and delta +inf) and far-travelled rays (large sides, where the chains' rounding drifts from
s + k * delta); the prefix estimates, which the kernels take from an approximate division, are
perturbed by -2..+2 so that the exact walk-up from a short prefix and the settle from S(0) after an
overshooting one both run."""
import math
import random

import numpy as np

f32 = np.float32
INF = float("inf")


def fadd(a, b):
    return f32(f32(a) + f32(b))


def fma(a, b, c):
    # the product of two binary32 values is exact in binary64; one more rounding than a true fused
    # multiply-add, which the candidate bound's margin covers
    return f32(float(a) * float(b) + float(c))


def fminf(a, b):
    if math.isnan(a):
        return b
    if math.isnan(b):
        return a
    return a if a <= b else b


def add_chain(s, d, k):
    for _ in range(k):
        s = fadd(s, d)
    return s


def literal(s, d, st, n):
    """Iterates the DDA step until some stepping axis has taken its n-th move."""
    s = list(s)
    moves = [0, 0, 0]
    while True:
        mn = fminf(fminf(s[0], s[1]), s[2])
        m = [s[a] == mn for a in range(3)]
        for a in range(3):
            if m[a]:
                s[a] = fadd(s[a], d[a])
                moves[a] += 1
        if any(m[a] and st[a] and moves[a] == n[a] for a in range(3)):
            return s, moves, m


def advance_axis(s, d, n, ts, err):
    if s > ts:
        return s, 0, False
    k = max(min(int(f32(f32(ts) - s) / d) + err, n - 2), 0)
    x = add_chain(s, d, k)
    if x > ts:
        k, x = 0, s
    y = fadd(x, d)
    while y <= ts and k + 1 < n:
        x, y, k = y, fadd(y, d), k + 1
    return y, k + 1, x == ts


def prefix_count(s, d, n, amin, err):
    if s > amin:
        return 0
    return max(min(int(f32(f32(amin) - s) / d) + err, n - 2), 0)


def finish_axis(s, h, k, d, n, ts, err):
    if h <= ts:
        x, y = h, fadd(h, d)
        while y <= ts and k + 1 < n:
            x, y, k = y, fadd(y, d), k + 1
        return y, k + 1, x == ts
    if k == 0:
        return s, 0, False
    return advance_axis(s, d, n, ts, err)


def crossing(s, d, n, errs):
    a = [fma(f32(n[i] - 1), d[i], s[i]) for i in range(3)]
    amin = fminf(fminf(a[0], a[1]), a[2])
    lim = fma(f32((max(n) + 2) * 2.0 ** -20), amin, amin)
    c = [bool(a[i] <= lim) for i in range(3)]
    k = [n[i] - 1 if c[i] else prefix_count(s[i], d[i], n[i], amin, errs[i]) for i in range(3)]
    h = [add_chain(s[i], d[i], k[i]) for i in range(3)]
    ts = fminf(fminf(h[0] if c[0] else f32(INF), h[1] if c[1] else f32(INF)),
               h[2] if c[2] else f32(INF))
    out = [finish_axis(s[i], h[i], k[i], d[i], n[i], ts, errs[i]) for i in range(3)]
    return [o[0] for o in out], [o[1] for o in out], [o[2] for o in out]


def random_case(rng):
    """Side distances, deltas, step signs and moves to the box face of one crossing."""
    st = [rng.choice((-1, 1)) for _ in range(3)]
    if rng.random() < 0.2:
        st[rng.randrange(3)] = 0
    travelled = rng.choice((1.0, 64.0, 1024.0, 30000.0))
    s, d, n = [], [], []
    for a in range(3):
        if st[a] == 0:
            s.append(f32(INF))
            d.append(f32(INF))
            n.append(0)
            continue
        da = f32(1.0 + rng.random() * rng.choice((0.5, 4.0, 60.0)))
        d.append(da)
        s.append(f32(travelled * rng.random() + float(da) * rng.random()))
        n.append(rng.randint(1, 64))
    if rng.random() < 0.25:  # ties: two axes with equal sides and deltas (diagonal rays)
        i = rng.randrange(3)
        j = (i + 1) % 3
        if st[i] and st[j]:
            s[j], d[j] = s[i], d[i]
    if not any(st):
        st[0], s[0], d[0], n[0] = 1, f32(0.5), f32(1.0), 3
    return s, d, st, n


def test_crossing_equals_the_iterated_step():
    rng = random.Random(20261204)
    for case in range(4000):
        s, d, st, n = random_case(rng)
        want = literal(s, d, st, n)
        errs = [rng.choice((-2, -1, 0, 0, 0, 1, 2)) for _ in range(3)]
        got = crossing(s, d, n, errs)
        for a in range(3):
            assert got[0][a] == want[0][a] or (math.isinf(got[0][a]) and math.isinf(want[0][a])), \
                (case, a, s, d, st, n, errs, got, want)
            assert got[1][a] == want[1][a], (case, a, s, d, st, n, errs, got, want)
            assert got[2][a] == want[2][a], (case, a, s, d, st, n, errs, got, want)


def test_crossing_with_exact_estimates_on_far_rays():
    # unperturbed estimates on rays far along (sides near 2^15-2^20), where chains of binary32
    # additions drift furthest from s + k * delta
    rng = random.Random(7)
    for case in range(1500):
        s, d, st, n = random_case(rng)
        s = [x if math.isinf(x) else f32(float(x) * 32.0 + 32768.0) for x in s]
        want = literal(s, d, st, n)
        got = crossing(s, d, n, [0, 0, 0])
        assert got[1] == want[1] and got[2] == want[2], (case, s, d, st, n, got, want)
        assert all(g == w or (math.isinf(g) and math.isinf(w)) for g, w in zip(got[0], want[0]))
