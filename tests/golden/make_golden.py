"""Generate the golden parity fixtures from the reference renderer itself.

The reference (renderer.cpp) is compiled by ``make -C oracle ref`` into
``oracle/_ref/mandelbrot.so`` with its release flags (no -march=native, hence
no compiler-chosen FMA: every double operation rounds on its own).  This
script runs every case of ``cases.py`` through that library's C ABI and
stores, per case, ``fixtures/<name>.npz`` with the float32 field, the uint32
iteration counts (escape index, cap for interior, 0 for NaN glitches) and,
for small cases, the six render planes.  Large cases store only SHA-256
digests and summary numbers in ``fixtures/index.json``.

Run here, where the reference sources exist:
    make -C oracle ref && python -m tests.golden.make_golden
"""

from __future__ import annotations

import json
import os
import sys

import numpy as np

from . import cases as case_defs
from .runner import _native, run_case, summary

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
FIXTURES = os.path.join(HERE, "fixtures")
REFERENCE_LIBRARY = os.path.join(ROOT, "oracle", "_ref", "mandelbrot.so")
PLANE_LIMIT = 64 * 36  # store the f64 planes only for cases this small


def main() -> int:
    native = _native()
    library = native.load(REFERENCE_LIBRARY)
    os.makedirs(FIXTURES, exist_ok=True)
    index = {"library": "oracle/_ref/mandelbrot.so (reference release build)", "cases": {}}
    all_cases = case_defs.parity_cases() + case_defs.alternate_cases()
    for case in all_cases:
        result = run_case(library, case)
        info = summary(result)
        index["cases"][case["name"]] = info
        if case.get("store") != "hash":
            arrays = {"field": result["field"], "counts": result["counts"]}
            if case["width"] * case["height"] <= PLANE_LIMIT:
                for key in ("orbit_iteration", "phase", "de_x", "de_y", "test1", "test2"):
                    arrays[key] = result[key]
            np.savez_compressed(os.path.join(FIXTURES, case["name"] + ".npz"), **arrays)
        print(f"{case['name']:28s} sum={info['count_sum']:>12d} nan={info['nan_pixels']:>5d} "
              f"range=[{info['count_min']},{info['count_max']}]")
    with open(os.path.join(FIXTURES, "index.json"), "w", encoding="ascii") as handle:
        json.dump(index, handle, indent=1, sort_keys=True)
        handle.write("\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
