"""The atlas KFP fixtures are the reference's own output.

The fixture file must hold every case of ``golden/kfp_atlas_cases.py``;
where the reference build exists (``oracle/_ref/mandelbrot.so``), a few
cases are coloured again and must equal the stored RGB bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from .golden import kfp_atlas_cases


def test_every_kfp_atlas_case_has_a_fixture():
    with np.load(kfp_atlas_cases.KFP_ATLAS_FIXTURE) as data:
        names = set(data.files)
    assert {c["name"] for c in kfp_atlas_cases.kfp_atlas_cases()} <= names


@pytest.mark.parametrize("name", ["tiles_feather0", "tiles_method4_feather6", "planes_atlas_centred",
                                  "planes_atlas_mixed_sets"])
def test_reference_reproduces_kfp_atlas_fixture(reference_library, name):
    case = next(c for c in kfp_atlas_cases.kfp_atlas_cases() if c["name"] == name)
    out = kfp_atlas_cases.run(reference_library, case)
    with np.load(kfp_atlas_cases.KFP_ATLAS_FIXTURE) as data:
        np.testing.assert_array_equal(out, data[name])
