"""GPU: deep views against an independent mpmath pixel oracle.

Parity with the reference cannot catch a mistake both perturbation designs
share, so, like the reference's own mpmath checks
(tests/test_native_abi.py:1522-1815), these views are compared with a direct
z^2 + c iteration at 40 + log10(zoom) digits (fixtures made by
tests/golden/make_mpmath_golden.py): counts equal and smooth values within
0.02 for the plain FP64 form and the floatexp form, at 1e12, 1e30, 1e60 and
1e100.
"""

from __future__ import annotations

import ctypes
import json
import os

import numpy as np
import pytest

from .conftest import FIXTURES
from .golden import cases as case_defs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

with open(os.path.join(FIXTURES, "mpmath_pixels.json"), encoding="ascii") as _handle:
    VIEWS = json.load(_handle)["views"]


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("view", VIEWS, ids=lambda v: v["name"])
def test_view_matches_mpmath(package, product, view, form):
    native = package.native
    with np.load(os.path.join(FIXTURES, "mpmath_pixels.npz")) as data:
        want = data[view["name"] + "_smooth"]
        want_counts = data[view["name"] + "_counts"]
    w, h, cap = view["width"], view["height"], view["max_iter"]
    zoom = case_defs.zoom_text(view["log10_zoom"]).encode()
    bits = case_defs.precision_bits(view["re"], view["im"], view["log10_zoom"])
    handle = native.create_reference(product, view["re"], view["im"], zoom, cap, bits, 32)
    field = torch.empty(w * h, dtype=torch.float32, device="cuda")
    counts = torch.empty(w * h, dtype=torch.int32, device="cuda")
    try:
        options = native.RenderOptions()
        status = product.fractal_gb300_render_reference_device(
            ctypes.c_void_p(field.data_ptr()), ctypes.c_void_p(counts.data_ptr()), w, h, zoom, ctypes.c_void_p(handle),
            cap, 3, 256, ctypes.byref(options), form, None)
        assert status == 0, native.last_error(product)
        torch.cuda.synchronize()
    finally:
        product.fractal_destroy_reference(handle)
    got = field.cpu().numpy().astype(np.float64)
    np.testing.assert_array_equal(counts.cpu().numpy().astype(np.uint32), want_counts)
    assert np.max(np.abs(got - want)) <= 0.02, np.max(np.abs(got - want))
