"""GPU: the no-allocation direct render against the regular device entry point.

fractal_gb300_render_direct_device_noalloc renders with a fixed scratch array
compiled into the library instead of allocated buffers.  Its pixels must
equal fractal_gb300_render_direct_device's bit for bit (the direct path's
parity bar), on two calls in a row that reuse the shared array, and fields
too large for the array must be refused without a launch.  The file name
makes pytest collect it last; it also passes alone in a fresh process.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

_ARGS = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
         ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
         ctypes.c_void_p]

VIEWS = [
    # (zoom, x, y, width, height, cap): an interior-heavy whole-set view, then
    # a deeper one of another size, so the second call rewrites the array.
    (b"1", b"-0.5", b"0.0", 640, 360, 3000),
    (b"4.5e5", b"-0.743643887037151", b"0.13182590420533", 480, 270, 8000),
]


def _bind(product):
    for name in ("fractal_gb300_render_direct_device_noalloc", "fractal_gb300_render_direct_device"):
        function = getattr(product, name)
        function.restype = ctypes.c_int
        function.argtypes = _ARGS


def _render(product, package, name, view, stream):
    zoom, x, y, w, h, cap = view
    field = torch.full((w * h,), -1.0, dtype=torch.float32, device="cuda")
    counts = torch.zeros((w * h,), dtype=torch.int32, device="cuda")
    options = package.native.RenderOptions()
    status = getattr(product, name)(field.data_ptr(), counts.data_ptr(), w, h, zoom, x, y, cap, 0, 0.0, 0.0,
                                    ctypes.addressof(options), stream)
    assert status == 0, package.native.last_error(product)
    return field, counts


def test_no_alloc_matches_device_entry_on_two_calls(product, package):
    _bind(product)
    stream = torch.cuda.Stream()
    results = []
    for view in VIEWS:  # two calls in a row on one stream, sharing the array
        results.append(_render(product, package, "fractal_gb300_render_direct_device_noalloc", view,
                               stream.cuda_stream))
    torch.cuda.synchronize()
    for view, (field, counts) in zip(VIEWS, results):
        want_field, want_counts = _render(product, package, "fractal_gb300_render_direct_device", view,
                                          stream.cuda_stream)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(counts.cpu().numpy(), want_counts.cpu().numpy())
        np.testing.assert_array_equal(field.cpu().numpy().view(np.uint32),
                                      want_field.cpu().numpy().view(np.uint32))


def test_no_alloc_rejects_fields_beyond_its_scratch(product, package):
    _bind(product)
    # 16352 + 1 columns and rows in total: one past the array's limit.  The
    # call must fail before any launch (the buffer is full size all the same).
    field = torch.empty((16000 * 353,), dtype=torch.float32, device="cuda")
    options = package.native.RenderOptions()
    status = product.fractal_gb300_render_direct_device_noalloc(
        field.data_ptr(), None, 16000, 353, b"1", b"-0.5", b"0.0", 100, 0, 0.0, 0.0,
        ctypes.addressof(options), None)
    assert status == 1
    message = package.native.last_error(product)
    assert "no-allocation" in message and "16352" in message, message
