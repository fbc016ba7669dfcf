"""Generate the seeded deep-zoom centres used by the parity tests and bench.

The reference bundles hand-picked centres only; the workloads here need
seeded Misiurewicz points instead.  A Misiurewicz point M(k, p) is a
parameter c whose critical orbit z_0 = 0, z_{n+1} = z_n^2 + c is strictly
preperiodic with preperiod k and period p:  z_{k+p} = z_k, while
z_{k-1+p} != z_{k-1} and z_{k+d} != z_k for every proper divisor d of p.
It lies on the boundary of the Mandelbrot set, so a deep view centred on it
keeps detail at every depth.

Method (seeded, deterministic):
  1. draw k ~ U{3..20}, p ~ U{1..8} and a start c0 in the upper half-plane;
  2. Newton on g(c) = z_{k+p}(c) - z_k(c) in double precision, with
     dz/dc carried alongside (d z_{n+1} = 2 z_n dz_n + 1);
  3. polish the converged root with Newton at the requested binary precision
     (mpmath, 400 or 1200 bits) and check the exact preperiod and period;
  4. reject and redraw on any failure.
The centres are printed as decimal strings of the requested length.

Julia constants for the mixed-formula batch are boundary points of the
Mandelbrot set found by bisection along a seeded ray (inside = critical
orbit bounded for the test budget), with |c| < 0.8.

Run:  python tests/golden/make_centres.py   (writes tests/golden/centres.json)
"""

from __future__ import annotations

import json
import math
import os
import sys

import mpmath
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _orbit_with_derivative(c: complex, steps: int):
    z = 0j
    dz = 0j
    zs = [z]
    dzs = [dz]
    for _ in range(steps):
        dz = 2.0 * z * dz + 1.0
        z = z * z + c
        zs.append(z)
        dzs.append(dz)
        if abs(z) > 1e150:
            return None, None
    return zs, dzs


def _newton_double(c: complex, k: int, p: int, iterations: int = 600):
    for _ in range(iterations):
        zs, dzs = _orbit_with_derivative(c, k + p)
        if zs is None:
            return None
        g = zs[k + p] - zs[k]
        dg = dzs[k + p] - dzs[k]
        if dg == 0:
            return None
        step = g / dg
        c = c - step
        if not (abs(c) < 4.0):
            return None
        if abs(step) < 1e-15:
            return c
    return None


def _mp_orbit(c, steps):
    z = mpmath.mpc(0)
    dz = mpmath.mpc(0)
    zs = [z]
    dzs = [dz]
    for _ in range(steps):
        dz = 2 * z * dz + 1
        z = z * z + c
        zs.append(z)
        dzs.append(dz)
    return zs, dzs


def misiurewicz_centre(seed: int, bits: int, digits: int):
    rng = np.random.default_rng(seed)
    for attempt in range(10_000):
        k = int(rng.integers(3, 21))
        p = int(rng.integers(1, 9))
        c0 = complex(rng.uniform(-2.0, 0.5), rng.uniform(0.02, 1.2))
        root = _newton_double(c0, k, p)
        if root is None or root.imag <= 1e-6:
            continue
        with mpmath.workprec(bits + 64):
            c = mpmath.mpc(root.real, root.imag)
            for _ in range(40):
                zs, dzs = _mp_orbit(c, k + p)
                g = zs[k + p] - zs[k]
                dg = dzs[k + p] - dzs[k]
                step = g / dg
                c = c - step
                if abs(step) < mpmath.mpf(2) ** (-(bits + 32)):
                    break
            zs, _ = _mp_orbit(c, k + p)
            tiny = mpmath.mpf(2) ** (-(bits - 16))
            loose = mpmath.mpf(10) ** -12
            if abs(zs[k + p] - zs[k]) > tiny:
                continue
            if abs(zs[k - 1 + p] - zs[k - 1]) < loose:
                continue  # smaller preperiod
            if any(abs(zs[k + d] - zs[k]) < loose for d in range(1, p) if p % d == 0):
                continue  # smaller period
            if any(abs(z) < loose for z in zs[1:]):
                continue  # a periodic centre, not a boundary point
            if c.imag <= 0:
                continue
            re = mpmath.nstr(c.real, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
            im = mpmath.nstr(c.imag, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
            return {
                "seed": seed,
                "attempt": attempt,
                "preperiod": k,
                "period": p,
                "bits": bits,
                "digits": digits,
                "re": re,
                "im": im,
            }
    raise RuntimeError("no Misiurewicz point found")


def nucleus_centre(seed: int, period: int, bits: int, digits: int):
    """Centre of a period-p hyperbolic component (z_p(c) = 0), found by
    Newton from a seeded start; its minibrot fills deep views with interior
    pixels, which exercises BLA, rebasing and long exact tails."""
    rng = np.random.default_rng(seed)
    for attempt in range(10_000):
        c0 = complex(rng.uniform(-1.9, 0.4), rng.uniform(0.02, 1.1))
        c = c0
        ok = False
        for _ in range(400):
            z, dz = 0j, 0j
            for _ in range(period):
                dz = 2.0 * z * dz + 1.0
                z = z * z + c
            if dz == 0 or abs(z) > 1e100:
                break
            step = z / dz
            c -= step
            if abs(c) > 2.5:
                break
            if abs(step) < 1e-15:
                ok = True
                break
        if not ok or c.imag <= 1e-4:
            continue
        with mpmath.workprec(bits + 64):
            cm = mpmath.mpc(c.real, c.imag)
            for _ in range(60):
                z, dz = mpmath.mpc(0), mpmath.mpc(0)
                for _ in range(period):
                    dz = 2 * z * dz + 1
                    z = z * z + cm
                step = z / dz
                cm = cm - step
                if abs(step) < mpmath.mpf(2) ** (-(bits + 32)):
                    break
            # exact period: no earlier return to zero
            z = mpmath.mpc(0)
            exact = True
            for k in range(1, period):
                z = z * z + cm
                if abs(z) < mpmath.mpf(10) ** -20:
                    exact = False
                    break
            if not exact:
                continue
            z, dz = mpmath.mpc(0), mpmath.mpc(0)
            for _ in range(period):
                dz = 2 * z * dz + 1
                z = z * z + cm
            size = float(1.0 / abs(dz) ** 2) if abs(dz) > 0 else 0.0
            re = mpmath.nstr(cm.real, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
            im = mpmath.nstr(cm.imag, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
            return {"seed": seed, "attempt": attempt, "period": period, "bits": bits, "digits": digits,
                    "size_estimate": size, "re": re, "im": im}
    raise RuntimeError("no nucleus found")


def nucleus_near(centre: dict, period: int, offset_log10: float, bits: int, digits: int):
    """Nucleus of a period-p minibrot on the spiral of a Misiurewicz point:
    Newton from the point shifted by 10^offset (1 + i).  Such minibrots sit
    at depth ~1e30 with long interior orbits, the regime where the BLA
    hierarchy, rebasing and replay do most of the work."""
    with mpmath.workprec(bits + 64):
        m = mpmath.mpc(mpmath.mpf(centre["re"]), mpmath.mpf(centre["im"]))
        cm = m + mpmath.mpf(10) ** offset_log10 * mpmath.mpc(1, 1)
        for _ in range(200):
            z, dz = mpmath.mpc(0), mpmath.mpc(0)
            for _ in range(period):
                dz = 2 * z * dz + 1
                z = z * z + cm
            step = z / dz
            cm = cm - step
            if abs(step) < mpmath.mpf(2) ** (-(bits + 16)):
                break
        else:
            raise RuntimeError("nucleus Newton did not converge")
        z, dz = mpmath.mpc(0), mpmath.mpc(0)
        for _ in range(period):
            dz = 2 * z * dz + 1
            z = z * z + cm
        re = mpmath.nstr(cm.real, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
        im = mpmath.nstr(cm.imag, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
        return {"period": period, "bits": bits, "digits": digits, "size_estimate": float(1 / abs(dz) ** 2),
                "distance_to_misiurewicz": float(abs(cm - m)), "re": re, "im": im}


def julia_fixed_point(c_re: str, c_im: str, digits: int = 120):
    """Repelling fixed point z* = (1 +- sqrt(1 - 4c)) / 2 (the larger-modulus
    root) of z^2 + c: the reference pipeline's deep Julia zoom target."""
    with mpmath.workdps(digits + 20):
        c = mpmath.mpc(mpmath.mpf(c_re), mpmath.mpf(c_im))
        root = mpmath.sqrt(1 - 4 * c)
        a, b = (1 + root) / 2, (1 - root) / 2
        z = a if abs(a) >= abs(b) else b
        re = mpmath.nstr(z.real, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
        im = mpmath.nstr(z.imag, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
        return {"re": re, "im": im, "c_re": c_re, "c_im": c_im}


def _alt_bounded(formula: str, c, budget: int) -> bool:
    z = mpmath.mpc(0)
    for _ in range(budget):
        if formula == "burning-ship":
            z = mpmath.mpc(abs(z.real), abs(z.imag)) ** 2 + c
        else:
            z = mpmath.conj(z) ** 2 + c
        if z.real * z.real + z.imag * z.imag > 4:
            return False
    return True


def alternate_boundary(formula: str, seed: int, digits: int = 40, budget: int = 1500):
    """A boundary point of the burning-ship or tricorn parameter set found by
    high-precision bisection along a seeded ray from an interior start."""
    rng = np.random.default_rng(seed)
    with mpmath.workdps(digits + 10):
        for _ in range(200):
            angle = rng.uniform(0.0, 2.0 * math.pi)
            start = mpmath.mpc(-0.2, 0.0) if formula == "tricorn" else mpmath.mpc(-0.3, -0.1)
            direction = mpmath.mpc(math.cos(angle), math.sin(angle))
            inner, outer = mpmath.mpf(0), mpmath.mpf(2)
            if not _alt_bounded(formula, start, budget) or _alt_bounded(formula, start + outer * direction, budget):
                continue
            for _ in range(int(digits * 3.4)):
                mid = (inner + outer) / 2
                if _alt_bounded(formula, start + mid * direction, budget):
                    inner = mid
                else:
                    outer = mid
            c = start + inner * direction
            re = mpmath.nstr(c.real, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
            im = mpmath.nstr(c.imag, digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
            return {"seed": seed, "angle": angle, "re": re, "im": im, "budget": budget}
    raise RuntimeError("no boundary point found")


def _bounded(c: complex, budget: int = 4000) -> bool:
    z = 0j
    for _ in range(budget):
        z = z * z + c
        if (z.real * z.real + z.imag * z.imag) > 4.0:
            return False
    return True


def julia_boundary_constant(seed: int):
    """A Mandelbrot-boundary parameter with |c| < 0.8 along a seeded ray."""
    rng = np.random.default_rng(seed)
    for _ in range(1000):
        angle = rng.uniform(0.0, 2.0 * math.pi)
        direction = complex(math.cos(angle), math.sin(angle))
        inner, outer = 0.0, 0.8
        if not _bounded(inner * direction) or _bounded(outer * direction):
            continue
        for _ in range(48):
            mid = 0.5 * (inner + outer)
            if _bounded(mid * direction):
                inner = mid
            else:
                outer = mid
        c = inner * direction
        return {"seed": seed, "angle": angle, "re": repr(c.real), "im": repr(c.imag)}
    raise RuntimeError("no Julia boundary constant found")


def _alt_orbit_jacobian(formula: str, cr, ci, steps: int):
    """Orbit of 0 under the burning-ship or tricorn map with the real
    Jacobian d(x, y)/d(cr, ci) carried along; stops early on escape."""
    x = y = xa = ya = xb = yb = mpmath.mpf(0)
    out = []
    for _ in range(steps):
        if formula == "burning-ship":
            sx, sy = (1 if x >= 0 else -1), (1 if y >= 0 else -1)
            ax, ay = abs(x), abs(y)
            x, y, xa, ya, xb, yb = (x * x - y * y + cr, 2 * ax * ay + ci,
                                    2 * x * xa - 2 * y * ya + 1, 2 * (sx * xa * ay + ax * sy * ya),
                                    2 * x * xb - 2 * y * yb, 2 * (sx * xb * ay + ax * sy * yb) + 1)
        else:
            x, y, xa, ya, xb, yb = (x * x - y * y + cr, -2 * x * y + ci,
                                    2 * x * xa - 2 * y * ya + 1, -2 * (xa * y + x * ya),
                                    2 * x * xb - 2 * y * yb, -2 * (xb * y + x * yb) + 1)
        out.append((x, y, xa, ya, xb, yb))
        if x * x + y * y > 1e6:
            break
    return out


def alternate_preperiodic(formula: str, seed: int, digits: int = 130):
    """A preperiodic (Misiurewicz-like) parameter of the burning-ship or
    tricorn map: z_{k+p} = z_k for seeded k ~ U{3..9}, p ~ U{1..4}, found by
    real 2x2 Newton from seeded starts, first at 60 digits, then polished at
    `digits`.  Views centred there show structure at every depth."""
    rng = np.random.default_rng(seed)

    def solve(c0, k, p, dps):
        with mpmath.workdps(dps + 20):
            cr, ci = mpmath.mpf(c0[0]), mpmath.mpf(c0[1])
            for it in range(120):
                o = _alt_orbit_jacobian(formula, cr, ci, k + p)
                if len(o) < k + p:
                    return None
                x1, y1, xa1, ya1, xb1, yb1 = o[k + p - 1]
                x0, y0, xa0, ya0, xb0, yb0 = o[k - 1]
                fx, fy = x1 - x0, y1 - y0
                j00, j01, j10, j11 = xa1 - xa0, xb1 - xb0, ya1 - ya0, yb1 - yb0
                det = j00 * j11 - j01 * j10
                if det == 0:
                    return None
                dr = (fx * j11 - fy * j01) / det
                di = (j00 * fy - j10 * fx) / det
                cr -= dr
                ci -= di
                if abs(dr) + abs(di) < mpmath.mpf(10) ** (-(dps + 5)):
                    return cr, ci, it
            return None

    for _ in range(2000):
        c0 = (rng.uniform(-1.9, 0.6), rng.uniform(-1.6, 0.6))
        k, p = int(rng.integers(3, 10)), int(rng.integers(1, 5))
        rough = solve(c0, k, p, 60)
        if rough is None or rough[2] >= 100 or abs(rough[0]) + abs(rough[1]) < 1e-3:
            continue
        if abs(abs(rough[0]) - 1) < 1e-9 or abs(abs(rough[1]) - 1) < 1e-9:
            continue  # rational corner points
        fine = solve((rough[0], rough[1]), k, p, digits)
        if fine is None:
            continue
        with mpmath.workdps(digits + 20):
            re = mpmath.nstr(fine[0], digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
            im = mpmath.nstr(fine[1], digits, strip_zeros=False, min_fixed=-mpmath.inf, max_fixed=mpmath.inf)
        return {"seed": seed, "preperiod": k, "period": p, "re": re, "im": im}
    raise RuntimeError("no preperiodic point found")


def add_deep_alternates(path: str) -> None:
    """Add 130-digit preperiodic burning-ship and tricorn parameters (views
    to 1e100 need more than 100 digits) to an existing centres.json."""
    with open(path, encoding="ascii") as handle:
        centres = json.load(handle)
    centres.pop("burning_ship_boundary_deep", None)
    centres.pop("tricorn_boundary_deep", None)
    centres["burning_ship_deep"] = alternate_preperiodic("burning-ship", seed=8301)
    centres["tricorn_deep"] = alternate_preperiodic("tricorn", seed=8302)
    with open(path, "w", encoding="ascii") as handle:
        json.dump(centres, handle, indent=1)
        handle.write("\n")


def add_deep_mandelbrot(path: str) -> None:
    """Add a 1060-digit Misiurewicz centre (3600-bit Newton) for views beyond
    the double exponent range (1e1000) to an existing centres.json."""
    with open(path, encoding="ascii") as handle:
        centres = json.load(handle)
    centres["field_e1000"] = misiurewicz_centre(seed=20243, bits=3600, digits=1060)
    with open(path, "w", encoding="ascii") as handle:
        json.dump(centres, handle, indent=1)
        handle.write("\n")


def main() -> int:
    if "--deep-alternates" in sys.argv:
        add_deep_alternates(os.path.join(HERE, "centres.json"))
        return 0
    if "--deep-mandelbrot" in sys.argv:
        add_deep_mandelbrot(os.path.join(HERE, "centres.json"))
        return 0
    centres = {
        # 640x360 at 1e30: 400-bit Newton, 120-digit strings.
        "field_640x360_e30": misiurewicz_centre(seed=20240, bits=400, digits=120),
        # FHD keyframe stack to 1e50: 1200-bit Newton, 360-digit strings.
        "fhd_stack_e50": misiurewicz_centre(seed=20241, bits=1200, digits=360),
        # 1e100 fields: 1200-bit Newton.
        "field_e100": misiurewicz_centre(seed=20242, bits=1200, digits=360),
        "julia_c": [julia_boundary_constant(seed=7000 + i) for i in range(4)],
        # Minibrot nuclei for BLA-heavy parity views.
        "nucleus_p34": nucleus_centre(seed=9100, period=34, bits=600, digits=180),
        "nucleus_p61": nucleus_centre(seed=9101, period=61, bits=600, digits=180),
    }
    centres.update({
        # Deep minibrots on the e100 point's spiral (BLA-heavy views).
        "deep_nucleus_p70": nucleus_near(centres["field_e100"], 70, -18.0, bits=700, digits=210),
        "deep_nucleus_p80": nucleus_near(centres["field_e100"], 80, -18.0, bits=700, digits=210),
        "julia_fixed_1": julia_fixed_point(centres["julia_c"][1]["re"], centres["julia_c"][1]["im"]),
        "julia_fixed_2": julia_fixed_point(centres["julia_c"][2]["re"], centres["julia_c"][2]["im"]),
        "burning_ship_boundary": alternate_boundary("burning-ship", seed=8101),
        "tricorn_boundary": alternate_boundary("tricorn", seed=8102),
    })
    path = os.path.join(HERE, "centres.json")
    with open(path, "w", encoding="ascii") as handle:
        json.dump(centres, handle, indent=1)
        handle.write("\n")
    for key, value in centres.items():
        if isinstance(value, dict):
            print(key, value.get("preperiod"), value.get("period"), value.get("size_estimate"),
                  value["re"][:24], value["im"][:24])
    return 0


if __name__ == "__main__":
    sys.exit(main())
