"""The committed golden fixtures are the reference's own output.

Re-runs every parity case through the reference renderer compiled from its
sources (oracle/_ref/mandelbrot.so, release flags) and requires bit-identical
fields and counts.  Skipped where the reference sources are absent.
"""

from __future__ import annotations

import numpy as np
import pytest

from .conftest import golden_arrays
from .golden import cases as case_defs
from .golden.runner import run_case, summary

CASES = case_defs.parity_cases()


@pytest.mark.parametrize("case", [c for c in CASES if c["width"] * c["height"] <= 30000],
                         ids=lambda c: c["name"])
def test_reference_reproduces_fixture(reference_library, golden_index, case):
    result = run_case(reference_library, case)
    assert summary(result) == golden_index[case["name"]]
    stored = golden_arrays(case["name"])
    if stored is not None:
        np.testing.assert_array_equal(result["counts"], stored["counts"])
        np.testing.assert_array_equal(result["field"].view(np.uint32), stored["field"].view(np.uint32))
