"""Aurora colour-pass parity cases (fractal_colourise, fractal_colourise_accents).

Stored parity fields and a seeded synthetic field (a smooth ramp over the
whole palette with NaN, +-inf, interior and negative samples) at caps that
select the small and the 65,536-entry palettes, under several phase / vocal
/ instrumental / pitch controls, with and without accents and an interior
colour.  ``run`` drives any library exporting the renderer.h ABI.
"""

from __future__ import annotations

import os

import numpy as np

from .runner import _native

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = os.path.join(HERE, "fixtures")
AURORA_FIXTURE = os.path.join(FIXTURES, "aurora.npz")

CONTROLS = [(0.3, 0.4, 0.7, 0.5), (0.0, 0.0, 0.0, 0.0), (0.91, 1.0, 0.15, 0.83)]
ACCENTS = np.array([250, 40, 90, 30, 200, 120, 10, 60, 240], dtype=np.uint8)


def synthetic(width: int, height: int, cap: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ramp = np.linspace(-0.02 * cap, 1.02 * cap, width * height, dtype=np.float64)
    field = (ramp + rng.normal(scale=0.5, size=ramp.size)).astype(np.float32)
    marks = rng.integers(0, field.size, size=64)
    field[marks[:16]] = np.nan
    field[marks[16:24]] = np.inf
    field[marks[24:32]] = -np.inf
    field[marks[32:48]] = np.float32(cap)
    return field


def aurora_cases() -> list[dict]:
    cases = []
    for name, cap in (("e30_160x90", 50_000), ("fhd_level05_128x72", 2_000), ("e100_bias_64x36", 200_000),
                      ("direct_julia_96x54", 4_000)):
        for i, controls in enumerate(CONTROLS):
            cases.append(dict(name=f"aurora_{name}_c{i}", field=name, cap=cap, controls=controls, accents=False))
    for cap in (300, 5_000, 16_384, 120_000):
        cases.append(dict(name=f"aurora_synthetic_cap{cap}", field=None, cap=cap, controls=CONTROLS[0],
                          accents=False))
        cases.append(dict(name=f"aurora_synthetic_cap{cap}_accents", field=None, cap=cap, controls=CONTROLS[2],
                          accents=True))
    return cases


def inputs(case):
    if case["field"] is None:
        return synthetic(317, 211, case["cap"], case["cap"]), 317, 211
    stored = np.load(os.path.join(FIXTURES, case["field"] + ".npz"))
    width, height = (int(v) for v in case["field"].rsplit("_", 1)[1].split("x"))
    return stored["field"], width, height


def run(library, case: dict) -> np.ndarray:
    native = _native()
    field, width, height = inputs(case)
    if case["accents"]:
        return native.colourise_accents(library, field, width, height, case["cap"], *case["controls"], ACCENTS,
                                        interior=(12, 34, 56))
    return native.colourise(library, field, width, height, case["cap"], *case["controls"])
