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
import json
import os
import subprocess
import sys

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


_FRESH = r"""
import ctypes, json, sys
sys.path.insert(0, ROOT)
import torch
from tests.conftest import load_package
package = load_package()
product = package.native.load(package.build(), gb300=True)
fn = product.fractal_gb300_render_direct_device_noalloc
fn.restype = ctypes.c_int
fn.argtypes = ARGS
w, h = 480, 270
field = torch.empty(w * h, dtype=torch.float32, device="cuda")
counts = torch.empty(w * h, dtype=torch.int32, device="cuda")
options = package.native.RenderOptions()
free = []
for _ in range(3):
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info()[0])
    status = fn(field.data_ptr(), counts.data_ptr(), w, h, b"1", b"-0.5", b"0.0", 2000, 0, 0.0, 0.0,
                ctypes.addressof(options), None)
    assert status == 0, package.native.last_error(product)
torch.cuda.synchronize()
free.append(torch.cuda.mem_get_info()[0])
steps = ctypes.c_ulonglong(0)
assert product.fractal_gb300_last_direct_steps(ctypes.byref(steps)) == 1
print("MESSAGE", package.native.last_error(product))
print("FREE", json.dumps(free))
"""


def test_no_alloc_calls_create_no_thread_runtime():
    """In a fresh process making only no-allocation calls: the device's free
    memory does not change from the second call on (the first call may load
    the module's array), and the thread never made its runtime (streams,
    counters, grow-only scratch): fractal_gb300_last_direct_steps reports
    that no direct batch has run on this thread."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    args = "[" + ", ".join("ctypes." + a.__name__ for a in _ARGS) + "]"
    code = "ROOT = %r\nARGS = None\n" % root + _FRESH.replace("fn.argtypes = ARGS", "fn.argtypes = " + args)
    result = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=root)
    assert result.returncode == 0, result.stderr[-2000:]
    lines = {line.split(" ", 1)[0]: line.split(" ", 1)[1] for line in result.stdout.splitlines()
             if line.startswith(("MESSAGE", "FREE"))}
    assert "no direct batch has run on this thread" in lines["MESSAGE"], lines
    free = json.loads(lines["FREE"])
    assert free[1] == free[2] == free[3], free


def test_last_direct_steps_after_a_no_alloc_call(product, package):
    """After an allocating direct render and then a no-allocation one on the
    same thread, the step counter refuses to report the allocating call's
    count as if it were the last launch's."""
    _bind(product)
    stream = torch.cuda.Stream()
    _render(product, package, "fractal_gb300_render_direct_device", VIEWS[1], stream.cuda_stream)
    steps = ctypes.c_ulonglong(0)
    assert product.fractal_gb300_last_direct_steps(ctypes.byref(steps)) == 0
    _render(product, package, "fractal_gb300_render_direct_device_noalloc", VIEWS[1], stream.cuda_stream)
    torch.cuda.synchronize()
    assert product.fractal_gb300_last_direct_steps(ctypes.byref(steps)) == 1
    assert "no-allocation" in package.native.last_error(product)
