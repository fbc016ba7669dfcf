"""GPU parity: the plain FP64 form against the reference's own output.

Every case of tests/golden/cases.py runs through the GB300 library's C ABI
(the same call sequence a ctypes caller of renderer.h makes).  The bar is the
reference release build's output, bit for bit: uint32 iteration counts
identical, float32 field identical (NaN glitch mask included).  The six
double render planes are compared where the fixture stores them:
orbit_iteration and test1/test2 exactly, phase and the analytic DE within
1e-12 relative (they pass through atan2/hypot/log, whose last bit differs
between CUDA's and glibc's libm).
"""

from __future__ import annotations

import numpy as np
import pytest

from .conftest import golden_arrays
from .golden import cases as case_defs
from .golden.runner import run_case, summary

pytestmark = pytest.mark.gpu

CASES = case_defs.parity_cases() + case_defs.alternate_cases()


def _field_bits(field):
    return np.ascontiguousarray(field, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_plain_form_matches_reference(product, golden_index, case):
    result = run_case(product, case)
    expected = golden_index[case["name"]]
    stored = golden_arrays(case["name"])
    if stored is None:
        got = summary(result)
        assert got["counts_sha256"] == expected["counts_sha256"], (got, expected)
        assert got["field_sha256"] == expected["field_sha256"], (got, expected)
        return
    counts = result["counts"]
    mismatch = np.count_nonzero(counts != stored["counts"])
    assert mismatch == 0, f"{mismatch} of {counts.size} counts differ"
    np.testing.assert_array_equal(np.isnan(result["field"]), np.isnan(stored["field"]))
    np.testing.assert_array_equal(_field_bits(result["field"]), _field_bits(stored["field"]))
    if "orbit_iteration" in stored:
        np.testing.assert_array_equal(result["orbit_iteration"], stored["orbit_iteration"])
        np.testing.assert_array_equal(result["test1"], stored["test1"])
        np.testing.assert_array_equal(result["test2"], stored["test2"])
        for key in ("phase", "de_x", "de_y"):
            np.testing.assert_allclose(result[key], stored[key], rtol=1e-12, atol=1e-300)


def test_stats_counters_match_reference_fields(product, package):
    """Device counters follow the reference's RenderStats field order; the
    logical iteration total plus series jumps equals the sum of counts for a
    strict render without glitches."""
    native = package.native
    case = next(c for c in CASES if c["name"] == "e30_160x90")
    product.fractal_set_stats_enabled(1)
    try:
        result = run_case(product, case)
        stats = native.stats(product)
    finally:
        product.fractal_set_stats_enabled(0)
    assert stats["pixels"] == case["width"] * case["height"]
    counts = result["counts"].astype(np.int64)
    assert stats["series_pixels"] == case["width"] * case["height"]
    # Each pixel starts at iteration 1 (or the series iteration) and ends at
    # its escape index.
    series_start = stats["series_jumps"] // max(1, stats["series_pixels"])
    assert stats["logical_iterations"] == int((counts - series_start).sum())


@pytest.mark.parametrize("name", ["fhd_level33_128x72", "deep_p80_e32_96x54", "deep_p70_e28_linear_96x54",
                                  "julia_fixed_1_e9_96x54", "burning-ship_e7_96x54", "tricorn_e12_64x36"])
def test_host_and_gpu_table_builders_agree(product, name):
    """The BLA hierarchies built on the GPU (default) and on the host use the
    same arithmetic; renders from either are bit-identical."""
    case = next(c for c in CASES if c["name"] == name)
    try:
        product.fractal_gb300_set_table_builder(0)
        host = run_case(product, case)
    finally:
        product.fractal_gb300_set_table_builder(1)
    device = run_case(product, case)
    np.testing.assert_array_equal(host["counts"], device["counts"])
    np.testing.assert_array_equal(_field_bits(host["field"]), _field_bits(device["field"]))
