"""The exact arithmetic the back-projection kernel relies on, checked in
NumPy against the reference's formulas (host-side restatements; the GPU parity
tests check the kernel itself bit for bit).

* Table index: the reference reads ker[clamp(roundf(fma(clamp(fl(Q - v), -2, 2),
  s, kc)), 0, T-1)] (gpuBackProject.cu:77-93).  The kernel reads entry
  min(floor(P * sat(fl(fma(Q, s/P, (h - v s)/P)))), T - 1), P a power of two
  >= T - 1, h = kc + 1/2, for voxel coordinates v >= 4.
* Brick intervals: the bricks of a row that meet the mask sphere form one x
  interval, computed from the integer (doubled-coordinate) box distance."""
import math

import numpy as np


def _f32(x):
    return np.asarray(x, np.float64).astype(np.float32).astype(np.float64)


def _roundf(x):
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def test_saturating_table_index_matches_reference_rule():
    rng = np.random.default_rng(5)
    for T in (501, 1000, 101, 513):
        kc = (T - 1) / 2.0
        s, h = kc / 2.0, kc + 0.5
        P = 512
        while P < T - 1:
            P *= 2
        for v in list(range(4, 12)) + list(rng.integers(12, 600, 8)):
            k = rng.integers(-300, T + 300, 4000)
            qb = (v + (k - h) / s).astype(np.float32)  # points near index boundaries and their neighbours
            Q = np.concatenate([_f32(v + rng.uniform(-4.2, 4.2, 8000)), _f32(qb),
                                _f32(np.nextafter(qb, np.float32(np.inf))), _f32(np.nextafter(qb, np.float32(-np.inf)))])
            Q = Q[np.abs(Q - v) <= 4.2]
            r = np.clip(_f32(Q - v), -2, 2)
            ref = np.clip(_roundf(_f32(r * s + kc)), 0, T - 1)
            sP, cP = s / P, (h - v * s) / P
            assert _f32(sP) == sP and _f32(cP) == cP  # the scaled constants are exact
            y = np.clip(_f32(Q * sP + cP), 0.0, 1.0)  # fma rounded once, then saturated
            got = np.minimum(np.floor(y * P), T - 1)
            assert np.array_equal(got, ref), (T, v)


def _brick_row(j, k, bricks_x, c, BZ, reach, BX=16, BY=8):
    d = lambda q, B: max(abs(2 * B * q + B - 1 - 2 * c) - (B - 1), 0)
    rem = 4 * (reach * reach + 1) - d(j, BY) ** 2 - d(k, BZ) ** 2
    if rem < 0:
        return set()
    t = math.isqrt(rem)
    lo = max(-((-(2 * c - 2 * (BX - 1) - t)) // (2 * BX)), 0)
    hi = min((2 * c + t) // (2 * BX), bricks_x - 1)
    return set(range(lo, hi + 1))


def _box_meets_sphere(i, j, k, c, BZ, reach, BX=16, BY=8):
    f = np.float32
    cx = max(abs(f(BX * i) + f(0.5 * (BX - 1)) - f(c)) - f(0.5 * (BX - 1)), f(0))
    cy = max(abs(f(BY * j) + f(0.5 * (BY - 1)) - f(c)) - f(0.5 * (BY - 1)), f(0))
    cz = max(abs(f(BZ * k) + f(0.5 * (BZ - 1)) - f(c)) - f(0.5 * (BZ - 1)), f(0))
    return not (f(cx * cx) + f(cy * cy) + f(cz * cz) > f(reach) * f(reach) + f(1))


def test_brick_row_intervals_match_the_box_test():
    for N in (2, 16, 21, 64, 128):
        M = 2 * N
        V, c, R = M + 6, (M + 6) // 2, M // 2 - 1
        for BZ in (12, 16):
            for reach in (R, R + 4):
                bx, by, bz = -(-V // 16), -(-V // 8), -(-V // BZ)
                for k in range(bz):
                    for j in range(by):
                        want = {i for i in range(bx) if _box_meets_sphere(i, j, k, c, BZ, reach)}
                        assert _brick_row(j, k, bx, c, BZ, reach) == want, (N, BZ, reach, j, k)
