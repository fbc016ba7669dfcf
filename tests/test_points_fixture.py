"""The point-render fixtures are the reference's own output.

Where the reference build exists (``oracle/_ref/mandelbrot.so``), two cheap
cases are rendered again and must equal the stored fixture bit for bit; the
fixture file must hold every case of ``golden/points_cases.py``.
"""

from __future__ import annotations

import numpy as np
import pytest

from .golden import points_cases


def test_every_point_case_has_a_fixture():
    with np.load(points_cases.POINTS_FIXTURE) as data:
        names = {key.split("/")[0] for key in data.files}
    assert {c["name"] for c in points_cases.point_cases()} <= names


@pytest.mark.parametrize("name", ["points_e30_fieldonly", "points_tricorn_e12"])
def test_reference_reproduces_point_fixture(reference_library, name):
    case = next(c for c in points_cases.point_cases() if c["name"] == name)
    result = points_cases.run(reference_library, case)
    with np.load(points_cases.POINTS_FIXTURE) as data:
        np.testing.assert_array_equal(result["field"].view(np.uint32), data[f"{name}/field"].view(np.uint32))


@pytest.mark.parametrize("case", [c for c in points_cases.point_cases()
                                  if c["formula"] == "mandelbrot" and "glitch" not in c["name"]],
                         ids=lambda c: c["name"])
def test_port_points_match_reference_fixture(oracle_port, case):
    """The oracle port's point renders (no exact repair) equal the reference
    on this host, planes included."""
    result = points_cases.run(oracle_port, case)
    with np.load(points_cases.POINTS_FIXTURE) as data:
        for key, value in result.items():
            np.testing.assert_array_equal(value, data[f"{case['name']}/{key}"])
