"""GPU: fractal_colourise_kfp_planes (the KFP colour pass driven by the
reference's render planes) against the reference's stored output.

Every case of ``golden/kfp_planes_cases.py`` -- stored orbit / phase /
distance-estimate / test planes of parity renders, bailout planes,
iteration + transition planes with hidden and shown glitches, the analytic
distance estimate, phase colour strength, both smoothing methods and
texture merging -- is
within +-1 per channel of the reference with >= 99.9 % of bytes exact (the
colour pass computes its transcendentals in FP32, the reference in FP64).
"""

from __future__ import annotations

import numpy as np
import pytest

from .golden import kfp_planes_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def planes_fixture():
    with np.load(kfp_planes_cases.KFP_PLANES_FIXTURE) as data:
        return {key: data[key] for key in data.files}


@pytest.mark.parametrize("case", kfp_planes_cases.kfp_planes_cases(), ids=lambda c: c["name"])
def test_kfp_planes_match_reference_within_one_lsb(product, planes_fixture, case):
    out = kfp_planes_cases.run(product, case)
    expected = planes_fixture[case["name"]]
    assert out.shape == expected.shape
    diff = np.abs(out.astype(np.int16) - expected.astype(np.int16))
    assert diff.max() <= 1, f"max channel difference {diff.max()} at {np.flatnonzero(diff > 1)[:8]}"
    assert np.mean(diff == 0) >= 0.999, f"only {np.mean(diff == 0):.5f} of bytes exact"


def test_kfp_planes_reject_short_texture_stride(product):
    """A texture stride below width * 3 fails with the reference's message
    and leaves the library usable."""
    import ctypes

    from .golden.runner import _native

    native = _native()
    case = next(c for c in kfp_planes_cases.kfp_planes_cases() if c["texture"] is not None)
    field, width, height, max_iter, options, planes, lut = kfp_planes_cases.inputs(case)
    rows, tw, th, _ = planes["texture"]
    struct = native.KfpPlanes()
    struct.struct_size = ctypes.sizeof(native.KfpPlanes)
    struct.version = 1
    struct.texture_rgb = rows.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    struct.texture_width, struct.texture_height, struct.texture_stride = tw, th, tw * 3 - 1
    field32 = np.ascontiguousarray(field, dtype=np.float32)
    out = np.empty(width * height * 3, dtype=np.uint8)
    status = product.fractal_colourise_kfp_planes(
        field32.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
        width, height, max_iter, 0.0, 0.0, 0.0, 0.5, ctypes.byref(options), ctypes.byref(struct),
        np.ascontiguousarray(lut).ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), lut.shape[0], 0)
    assert status != 0
    assert b"invalid native KFP colour" in product.fractal_last_error()
    again = kfp_planes_cases.run(product, case)
    assert again.shape == out.shape
