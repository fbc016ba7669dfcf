"""Host side of the KFP colour path: the LUT builder and the options block.

The LUT fixtures were built by the reference pipeline's own Python
(visualizer._kfp_palette_lut) for every named recipe; the restatement here
must reproduce them byte for byte.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

from .conftest import FIXTURES
from .golden import cases as case_defs


@pytest.fixture(scope="module")
def luts():
    with np.load(os.path.join(FIXTURES, "kfp_luts.npz")) as data:
        return {key: data[key] for key in data.files}


def test_lut_matches_reference_pipeline(package, luts):
    for name, expected in luts.items():
        got = package.kfp.palette_lut(package.kfp.recipe(name))
        np.testing.assert_array_equal(got, expected, err_msg=name)


def test_lut_known_answers(package):
    kfp = package.kfp
    # Two stops: entry 0 is the first stop, the half-way entry is their mean
    # (sin(0) = 0 -> fraction 1/2), and the table wraps back toward stop 0.
    profile = kfp.KfpProfile(stops=((0, 0, 0), (200, 100, 50)))
    lut = kfp.palette_lut(profile, size=8)
    assert tuple(lut[0]) == (0, 0, 0)
    assert tuple(lut[2]) == (100, 50, 25)
    assert tuple(lut[4]) == (200, 100, 50)
    assert lut[6][0] == 100 and lut[7][0] < lut[6][0]


def test_kfp_triplet_byte_order(package):
    kfp = package.kfp
    text = "Colors: 10,20,30,40,50,60\nColorMethod: 7\nDifferences: 3\nSlopes: 1\nIterDiv: 0.01\n"
    profile = kfp.parse_kfp(text)
    assert profile.stops == ((30, 20, 10), (60, 50, 40))
    assert profile.color_method == 7 and profile.slopes and profile.iter_div == 0.01
    assert kfp.with_relief(profile, False).slopes is False


def test_options_block(package):
    native = package.native
    kfp = package.kfp
    o = kfp.options(kfp.KALLES_DEFAULT, field_bias=12.5)
    assert o.struct_size == ctypes.sizeof(native.KfpOptions)
    assert o.version == 3
    assert (o.color_method, o.differences, o.slopes, o.smooth) == (7, 3, 1, 1)
    assert o.field_bias == 12.5
    with pytest.raises(ValueError):
        kfp.options(kfp.KALLES_DEFAULT, field_bias=-1.0)


def test_every_kfp_case_has_a_fixture():
    with np.load(os.path.join(FIXTURES, "kfp_rgb.npz")) as data:
        names = set(data.files)
    assert {c["name"] for c in case_defs.kfp_cases()} <= names
