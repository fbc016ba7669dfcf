"""The KFP plane-path fixtures are the reference's own output.

The fixture file must hold every case of ``golden/kfp_planes_cases.py``;
where the reference build exists (``oracle/_ref/mandelbrot.so``), a few
cases are coloured again and must equal the stored RGB bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from .golden import kfp_planes_cases


def test_every_kfp_planes_case_has_a_fixture():
    with np.load(kfp_planes_cases.KFP_PLANES_FIXTURE) as data:
        names = set(data.files)
    assert {c["name"] for c in kfp_planes_cases.kfp_planes_cases()} <= names


def test_hidden_glitches_differ_from_shown():
    """The hidden-glitch case paints the negative-transition pixels black."""
    with np.load(kfp_planes_cases.KFP_PLANES_FIXTURE) as data:
        shown = data["planes_iteration_glitches_shown_e100_nobla"].reshape(-1, 3)
        hidden = data["planes_iteration_glitches_hidden_e100_nobla"].reshape(-1, 3)
    changed = np.any(shown != hidden, axis=1)
    assert changed.any()
    assert np.all(hidden[changed] == 0)


@pytest.mark.parametrize("name", ["planes_differences7_odd_37x23", "planes_phase_e100_nobla",
                                  "planes_iteration_glitches_hidden_e100_nobla", "planes_texture_iteration_e100_nobla"])
def test_reference_reproduces_kfp_planes_fixture(reference_library, name):
    case = next(c for c in kfp_planes_cases.kfp_planes_cases() if c["name"] == name)
    out = kfp_planes_cases.run(reference_library, case)
    with np.load(kfp_planes_cases.KFP_PLANES_FIXTURE) as data:
        np.testing.assert_array_equal(out, data[name])
