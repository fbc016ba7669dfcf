"""CPU: the atlas helpers in atlas.py against the reference pipeline's own.

atlas.py restates the parts of visualizer.py that decide what the renderer
is asked for: the iteration cap per depth (max_iterations,
visualizer.py:6958-6979), the keyframe ladder (_atlas_geometry, :7628-7661),
the BLA input-radius tiers (_native_reference_tier_logs, :6409-6481), the
tier a keyframe selects (_select_native_reference, :6484-6510), the MPFR
precision (_native_precision_bits, :5025-5036) and the zoom string
(_zoom_text, :5118-5124).  On seeded inputs each must return exactly what
the reference's function returns.  Runs where the reference checkout is
present (it is imported read-only); skipped elsewhere.
"""

from __future__ import annotations

import math
import os
import sys

import numpy as np
import pytest

from .conftest import REFERENCE_SOURCES, load_package


@pytest.fixture(scope="module")
def visualizer():
    if not os.path.isfile(os.path.join(REFERENCE_SOURCES, "visualizer.py")):
        pytest.skip("reference sources are not present on this machine")
    sys.path.insert(0, REFERENCE_SOURCES)
    try:
        import visualizer as module  # noqa: PLC0415  (reference pipeline, read-only)
    finally:
        sys.path.remove(REFERENCE_SOURCES)
    return module


@pytest.fixture(scope="module")
def atlas():
    return load_package().atlas


def test_max_iterations(visualizer, atlas):
    rng = np.random.default_rng(11)
    for _ in range(500):
        log_zoom = float(rng.uniform(0.0, 320.0))
        base = int(rng.integers(64, 5000))
        per_decade = int(rng.integers(0, 5000))
        cap = int(rng.integers(base, 2_000_000))
        assert atlas.max_iterations(log_zoom, base, per_decade, cap) == \
            visualizer.max_iterations(log_zoom, base, per_decade, cap)


def test_atlas_geometry(visualizer, atlas):
    rng = np.random.default_rng(12)
    for _ in range(300):
        lo = float(rng.uniform(0.0, 50.0))
        zooms = np.sort(rng.uniform(lo, lo + rng.uniform(0.5, 200.0), int(rng.integers(2, 50))))
        factor = float(rng.choice([2.0, 4.0, 8.0, 16.0, float(rng.uniform(1.2, 20.0))]))
        assert atlas.atlas_geometry(zooms, factor) == visualizer._atlas_geometry(zooms, factor)


def test_reference_tiers_and_selection(visualizer, atlas):
    rng = np.random.default_rng(13)
    for _ in range(300):
        maximum = float(rng.uniform(0.0, 300.0))
        step = float(rng.choice([math.log10(8.0), math.log10(4.0), math.log10(2.0)])) if rng.random() < 0.7 else None
        tiers = atlas.reference_tier_logs(maximum, step)
        assert tiers == visualizer._native_reference_tier_logs(maximum, step)
        references = [(t, f"tier{t:.3f}") for t in tiers]
        for _ in range(10):
            log_zoom = float(rng.uniform(0.0, maximum + 5.0))
            margin = float(rng.choice([0.0, 0.5, 2.0]))
            assert atlas.select_reference(references, log_zoom, margin) == \
                visualizer._select_native_reference(references, log_zoom, margin)


def test_precision_and_zoom_text(visualizer, atlas):
    rng = np.random.default_rng(14)
    for _ in range(300):
        digits = int(rng.integers(1, 400))
        x = "-0." + "".join(str(int(d)) for d in rng.integers(0, 10, digits))
        y = "0." + "".join(str(int(d)) for d in rng.integers(0, 10, int(rng.integers(1, 400))))
        log_zoom = float(rng.uniform(0.0, 300.0))
        assert atlas.precision_bits(x, y, log_zoom) == visualizer._native_precision_bits(x, y, log_zoom)
        assert atlas.zoom_text(log_zoom) == visualizer._zoom_text(log_zoom)
