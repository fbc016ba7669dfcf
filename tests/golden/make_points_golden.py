"""Generate ``fixtures/points.npz``: every case of ``points_cases.py`` through
the reference renderer's own fractal_render_points[_ex_planes].

The reference is the release build ``oracle/_ref/mandelbrot.so`` (see
``make_golden.py``); per case the float32 field and, for planes cases, the
six render planes are stored under ``<case>/<key>``.

Run here, where the reference sources exist:
    make -C oracle ref && python -m tests.golden.make_points_golden
"""

from __future__ import annotations

import os
import sys
import time

import numpy as np

from . import points_cases
from .make_golden import REFERENCE_LIBRARY
from .runner import _native


def main() -> int:
    native = _native()
    library = native.load(REFERENCE_LIBRARY)
    arrays = {}
    for case in points_cases.point_cases():
        started = time.perf_counter()
        result = points_cases.run(library, case)
        for key, value in result.items():
            arrays[f"{case['name']}/{key}"] = value
        field = result["field"]
        print(f"{case['name']:28s} n={field.size} nan={int(np.isnan(field).sum())} "
              f"range=[{np.nanmin(field):.2f}, {np.nanmax(field):.2f}] {time.perf_counter() - started:.1f} s")
    np.savez_compressed(points_cases.POINTS_FIXTURE, **arrays)
    print(f"wrote {os.path.relpath(points_cases.POINTS_FIXTURE)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
