"""Generate ``fixtures/aurora.npz``: every case of ``aurora_cases.py``
through the reference's own fractal_colourise[_accents] (release build
``oracle/_ref/mandelbrot.so``).

Run here, where the reference sources exist:
    make -C oracle ref && python -m tests.golden.make_aurora_golden
"""

from __future__ import annotations

import os
import sys

import numpy as np

from . import aurora_cases
from .make_golden import REFERENCE_LIBRARY
from .runner import _native


def main() -> int:
    native = _native()
    library = native.load(REFERENCE_LIBRARY)
    outputs = {}
    for case in aurora_cases.aurora_cases():
        out = aurora_cases.run(library, case)
        outputs[case["name"]] = out
        print(f"{case['name']:40s} mean={out.mean():7.2f}")
    np.savez_compressed(aurora_cases.AURORA_FIXTURE, **outputs)
    print(f"wrote {os.path.relpath(aurora_cases.AURORA_FIXTURE)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
