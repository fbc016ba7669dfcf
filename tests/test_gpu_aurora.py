"""GPU: the aurora colour pass (fractal_colourise, fractal_colourise_accents)
against the reference's stored RGB, bit for bit: stored parity fields and a
synthetic ramp with NaN, +-inf, interior and negative samples, at caps that
select the small and the 65,536-entry palettes, under several controls,
with accents and an interior colour."""

from __future__ import annotations

import numpy as np
import pytest

from .golden import aurora_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def aurora_fixture():
    with np.load(aurora_cases.AURORA_FIXTURE) as data:
        return {key: data[key] for key in data.files}


@pytest.mark.parametrize("case", aurora_cases.aurora_cases(), ids=lambda c: c["name"])
def test_aurora_matches_reference(product, aurora_fixture, case):
    out = aurora_cases.run(product, case)
    expected = aurora_fixture[case["name"]]
    mismatch = np.flatnonzero(out != expected)
    assert mismatch.size == 0, f"{mismatch.size} bytes differ, first at {mismatch[:8]}"
