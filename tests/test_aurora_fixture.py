"""The aurora fixtures are the reference's own output: every case of
``golden/aurora_cases.py`` is stored, and where the reference build exists
two cases are coloured again and must match bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

from .golden import aurora_cases


def test_every_aurora_case_has_a_fixture():
    with np.load(aurora_cases.AURORA_FIXTURE) as data:
        names = set(data.files)
    assert {c["name"] for c in aurora_cases.aurora_cases()} <= names


@pytest.mark.parametrize("name", ["aurora_e30_160x90_c2", "aurora_synthetic_cap120000_accents"])
def test_reference_reproduces_aurora_fixture(reference_library, name):
    case = next(c for c in aurora_cases.aurora_cases() if c["name"] == name)
    out = aurora_cases.run(reference_library, case)
    with np.load(aurora_cases.AURORA_FIXTURE) as data:
        np.testing.assert_array_equal(out, data[name])
