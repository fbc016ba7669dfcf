"""Independent high-precision pixel oracle for deep views (mpmath).

The GB300 library and the reference share the perturbation design, so a
mistake common to both would pass every parity test.  Following the
reference's own mpmath checks (tests/test_native_abi.py:1522-1815), this
script iterates z <- z^2 + c directly in mpmath at 40 + log10(zoom) digits
for every pixel of a few small views of seeded centres (pixel geometry of
the renderer: height span 2.8 / zoom, pixel centres at
(i - (n - 1) / 2) * span / n) and stores the smooth escape value
n + 1 - log2(ln|z|) (renderer.cpp:8170-8181, counted from the escape index
n) and the escape index, or the cap for pixels still bounded.

Run here (needs mpmath; the GPU host only reads the fixture):
    python -m tests.golden.make_mpmath_golden
"""

from __future__ import annotations

import json
import os

import mpmath
import numpy as np

from . import cases as case_defs

HERE = os.path.dirname(os.path.abspath(__file__))
OUTPUT = os.path.join(HERE, "fixtures", "mpmath_pixels.npz")

# (name, centre key, log10 zoom, width, height, cap)
VIEWS = [
    ("e12_6x6", "field_640x360_e30", 12.0, 6, 6, 4000),
    ("e30_4x4", "field_640x360_e30", 30.0, 4, 4, 20000),
    ("e60_4x4", "field_e100", 60.0, 4, 4, 40000),
    ("e100_4x4", "field_e100", 100.0, 4, 4, 60000),
]


def views():
    c = case_defs.centres()
    return [dict(name=name, re=c[key]["re"], im=c[key]["im"], log10_zoom=z, width=w, height=h, max_iter=cap)
            for name, key, z, w, h, cap in VIEWS]


def render(view) -> tuple[np.ndarray, np.ndarray]:
    w, h, cap = view["width"], view["height"], view["max_iter"]
    with mpmath.workdps(int(40 + view["log10_zoom"])):
        cr, ci = mpmath.mpf(view["re"]), mpmath.mpf(view["im"])
        # The decimal zoom string the renderer parses.
        zoom = mpmath.mpf(case_defs.zoom_text(view["log10_zoom"]))
        span_h = mpmath.mpf("2.8") / zoom
        span_w = span_h * w / h
        smooth = np.zeros(w * h)
        counts = np.zeros(w * h, dtype=np.uint32)
        for py in range(h):
            yo = (mpmath.mpf(h - 1) / 2 - py) * span_h / h
            for px in range(w):
                xo = (mpmath.mpf(px) - mpmath.mpf(w - 1) / 2) * span_w / w
                c = mpmath.mpc(cr + xo, ci + yo)
                z = mpmath.mpc(0)
                value, count = float(cap), cap
                for n in range(cap):
                    z = z * z + c
                    m2 = z.real * z.real + z.imag * z.imag
                    if m2 > 4:
                        value = float(n + 1 - mpmath.log(mpmath.log(mpmath.sqrt(m2))) / mpmath.log(2))
                        count = n + 1
                        break
                smooth[py * w + px] = value
                counts[py * w + px] = count
    return smooth, counts


def main() -> int:
    arrays = {}
    for view in views():
        smooth, counts = render(view)
        arrays[view["name"] + "_smooth"] = smooth
        arrays[view["name"] + "_counts"] = counts
        print(view["name"], int(counts.min()), int(counts.max()))
    np.savez_compressed(OUTPUT, **arrays)
    with open(OUTPUT.replace(".npz", ".json"), "w", encoding="ascii") as handle:
        json.dump({"views": views()}, handle, indent=1)
        handle.write("\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
