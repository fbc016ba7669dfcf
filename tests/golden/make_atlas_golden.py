"""Generate ``fixtures/atlas.npz``: every case of ``atlas_cases.py`` run
through the reference renderer's own atlas entry points.

The reference is the release build ``oracle/_ref/mandelbrot.so`` (see
``make_golden.py``); its outputs are stored per case name (float32 frames for
the scalar compositor, RGB8 for the colour paths).

Run here, where the reference sources exist:
    make -C oracle ref && python -m tests.golden.make_atlas_golden
"""

from __future__ import annotations

import os
import sys

import numpy as np

from . import atlas_cases
from .make_golden import REFERENCE_LIBRARY
from .runner import _native


def main() -> int:
    native = _native()
    library = native.load(REFERENCE_LIBRARY)
    outputs = {}
    for case in atlas_cases.CASES:
        out = atlas_cases.run(library, case)
        outputs[case["name"]] = out
        finite = out[np.isfinite(out)] if out.dtype == np.float32 else out
        print(f"{case['name']:28s} {out.dtype} n={out.size} mean={float(finite.mean()):.4f}")
    np.savez_compressed(atlas_cases.ATLAS_FIXTURE, **outputs)
    print(f"wrote {os.path.relpath(atlas_cases.ATLAS_FIXTURE)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
