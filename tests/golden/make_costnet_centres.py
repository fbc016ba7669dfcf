"""Generate the seeded centres of the tile-cost network's training fields.

200 Misiurewicz points (preperiod ~U{3..20}, period ~U{1..8}, upper
half-plane), found by the same seeded Newton method as the parity centres
(tests/golden/make_centres.py: double-precision Newton, polished with mpmath
at 400 bits, exact preperiod/period checked) and written as 120-digit
decimals to fractal-audio-viz_gb300/costnet_centres.json, which the package
reads.  Needs mpmath; the GPU host only reads the JSON.

Run:  python tests/golden/make_costnet_centres.py
"""

from __future__ import annotations

import importlib.util
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
MAKER = os.path.join(HERE, "make_centres.py")
OUTPUT = os.path.join(os.path.dirname(os.path.dirname(HERE)), "fractal-audio-viz_gb300", "costnet_centres.json")


def main(count: int = 200, first_seed: int = 50_000) -> None:
    spec = importlib.util.spec_from_file_location("make_centres", MAKER)
    maker = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(maker)
    centres = [maker.misiurewicz_centre(first_seed + i, 400, 120) for i in range(count)]
    with open(OUTPUT, "w", encoding="ascii") as handle:
        json.dump({"method": "seeded Misiurewicz Newton, 400 bits, 120 digits", "centres": centres}, handle,
                  indent=1)


if __name__ == "__main__":
    main()
