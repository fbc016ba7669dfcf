"""Generate ``fixtures/kfp_planes.npz``: every case of ``kfp_planes_cases.py``
through the reference's own fractal_colourise_kfp_planes (release build
``oracle/_ref/mandelbrot.so``).

Run here, where the reference sources exist:
    make -C oracle ref && python -m tests.golden.make_kfp_planes_golden
"""

from __future__ import annotations

import os
import sys

import numpy as np

from . import kfp_planes_cases
from .make_golden import REFERENCE_LIBRARY
from .runner import _native


def main() -> int:
    native = _native()
    library = native.load(REFERENCE_LIBRARY)
    outputs = {}
    for case in kfp_planes_cases.kfp_planes_cases():
        out = kfp_planes_cases.run(library, case)
        outputs[case["name"]] = out
        print(f"{case['name']:48s} mean={out.mean():7.2f}")
    np.savez_compressed(kfp_planes_cases.KFP_PLANES_FIXTURE, **outputs)
    print(f"wrote {os.path.relpath(kfp_planes_cases.KFP_PLANES_FIXTURE)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
