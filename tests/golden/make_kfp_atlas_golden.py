"""Generate ``fixtures/kfp_atlas.npz``: every case of ``kfp_atlas_cases.py``
through the reference's own fractal_atlas_colourise_kfp[_planes] (release
build ``oracle/_ref/mandelbrot.so``).

Run here, where the reference sources exist:
    make -C oracle ref && python -m tests.golden.make_kfp_atlas_golden
"""

from __future__ import annotations

import os
import sys

import numpy as np

from . import kfp_atlas_cases
from .make_golden import REFERENCE_LIBRARY
from .runner import _native


def main() -> int:
    native = _native()
    library = native.load(REFERENCE_LIBRARY)
    outputs = {}
    for case in kfp_atlas_cases.kfp_atlas_cases():
        out = kfp_atlas_cases.run(library, case)
        outputs[case["name"]] = out
        print(f"{case['name']:40s} n={out.size // 3:6d} mean={out.mean():7.2f}")
    np.savez_compressed(kfp_atlas_cases.KFP_ATLAS_FIXTURE, **outputs)
    print(f"wrote {os.path.relpath(kfp_atlas_cases.KFP_ATLAS_FIXTURE)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
