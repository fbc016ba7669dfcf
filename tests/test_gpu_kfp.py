"""GPU: the KFP colour kernel against the reference's RGB8, +-1 LSB.

Each case colours a stored reference field with a named recipe through
fractal_colourise_kfp (the renderer.h ABI).  The bar: every channel within
+-1 of the reference output; the fraction of exactly equal bytes is also
required to stay above 99.9 %.
"""

from __future__ import annotations

import os

import numpy as np
import pytest

from .conftest import FIXTURES, golden_arrays
from .golden import cases as case_defs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def expected_rgb():
    with np.load(os.path.join(FIXTURES, "kfp_rgb.npz")) as data:
        return {key: data[key] for key in data.files}


def test_kfp_matches_reference_within_one_lsb(product, package, expected_rgb):
    kfp = package.kfp
    total = 0
    exact = 0
    worst = {}
    for case in case_defs.kfp_cases():
        field_case = next(c for c in case_defs.parity_cases() if c["name"] == case["field"])
        field = golden_arrays(case["field"])["field"]
        got = kfp.colourise(product, field, field_case["width"], field_case["height"], case["max_iter"],
                            kfp.recipe(case["recipe"]), field_bias=case["field_bias"])
        want = expected_rgb[case["name"]]
        diff = np.abs(got.astype(np.int16) - want.astype(np.int16))
        worst[case["name"]] = int(diff.max())
        total += diff.size
        exact += int((diff == 0).sum())
    bad = {k: v for k, v in worst.items() if v > 1}
    assert not bad, bad
    assert exact / total > 0.999, exact / total


@pytest.mark.parametrize("divisor", [255.0, 640.0, 100.0, 6.0, float(np.float32(np.pi) / np.float32(2.0))])
def test_constant_division_equals_ieee_division(product, divisor):
    """The KFP pass divides by its constants with a rounded-reciprocal
    product and one FMA correction; for every one of the 2^32 float inputs
    the quotient equals IEEE division bit for bit."""
    import ctypes

    mismatches = ctypes.c_ulonglong(99)
    assert product.fractal_gb300_check_division(divisor, ctypes.byref(mismatches)) == 0
    assert mismatches.value == 0
