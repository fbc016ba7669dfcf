"""CPU: the integer escape rule of the direct queue against IEEE addition.

render_direct.cu decides m2 > R^2 with m2 = RN(zr^2 + zi^2) on the bit
patterns of the two squares, without an FP64 add (sum_exceeds).  This file
restates that rule in Python integers and checks it against numpy's float64
addition on random squares, on sums within a few ulps of R^2 (both escape
radii), and on the exact rounding midpoints where ties-to-even decide.
"""

from __future__ import annotations

import numpy as np

MANT = (1 << 52) - 1


def bits(x: float) -> int:
    return int(np.float64(x).view(np.uint64))


def sum_exceeds(a: int, b: int, r2: int) -> bool:
    mag = (1 << 63) - 1
    a &= mag
    b &= mag
    if a < b:
        a, b = b, a
    if a > r2:
        return True
    if a <= r2 - (1 << 52):
        return False
    er = r2 >> 52
    mr = (r2 & MANT) | (1 << 52)
    ea = a >> 52
    big = ((a & MANT) | (1 << 52)) << (ea - er + 1)
    eb = b >> 52
    mb = b & MANT
    if eb == 0:
        eb = 1
    else:
        mb |= 1 << 52
    shift = eb - er + 1
    below = False
    if shift >= 0:
        small = mb << shift
    elif shift > -64:
        small = mb >> -shift
        below = (mb & ((1 << -shift) - 1)) != 0
    else:
        small = 0
        below = mb != 0
    total = big + small
    midpoint = 2 * mr + 1
    if total != midpoint:
        return total > midpoint
    return below or (mr & 1) != 0


def reference(a: float, b: float, r2: float) -> bool:
    m2 = np.float64(a) + np.float64(b)
    return bool(m2 > r2 or not np.isfinite(m2))


def test_rule_matches_float64_addition():
    rng = np.random.default_rng(3)
    for r2 in (4.0, 1.0e8):
        cases = []
        for _ in range(20000):
            x = rng.uniform(-1.2, 1.2) * np.sqrt(r2)
            y = rng.uniform(-1.2, 1.2) * np.sqrt(r2)
            cases.append((x * x, y * y))
        # sums within a few ulps of R^2
        ulp = np.spacing(np.float64(r2))
        for _ in range(20000):
            a = rng.uniform(0.0, r2)
            b = r2 - a + rng.integers(-4, 5) * ulp * rng.random()
            if b >= 0:
                cases.append((a, b))
        # exact midpoints above R^2 and their neighbours
        for k in range(1, 60):
            a = np.float64(r2) - np.ldexp(1.0, -k) * r2 / 4
            b = np.float64(r2) + ulp / 2 - a
            for db in (-1, 0, 1):
                bb = np.nextafter(b, np.inf) if db > 0 else (np.nextafter(b, -np.inf) if db < 0 else b)
                if bb >= 0:
                    cases.append((a, bb))
        cases += [(np.inf, 0.0), (np.nan, 1.0), (0.0, 0.0), (r2, 0.0), (r2 / 2, r2 / 2), (5e-324, r2)]
        for a, b in cases:
            assert sum_exceeds(bits(a), bits(b), bits(r2)) == reference(a, b, r2), (a, b, r2)
