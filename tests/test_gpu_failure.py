"""GPU: the bounded waits and budgets report instead of hanging.

* The per-pixel time budget (the reference's opt-in deadline,
  tests/test_native_abi.py:638-675): a pathological deep cell -- all
  interior, no BLA, no cycle detection, cap 30,000 -- with a 1 ms budget
  returns status 0, promptly, with its unfinished pixels NaN and every
  finished pixel equal to the unbudgeted render's.
* Extreme zoom (tests/test_native_abi.py:713-734): a reference prepared at
  1e6 renders 1e100 and 1e4000 fields that are finite everywhere.
* The direct queue's spill wait: with the test hook, spilled pixels are
  written but never published and the consumers' wait is bounded at 1,000
  polls; the kernel ends, and fractal_gb300_last_direct_steps reports the
  queue error.  The failure is made by data; nothing faults or traps.
"""

from __future__ import annotations

import ctypes
import time

import numpy as np
import pytest

from .golden import cases as case_defs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_time_budget_marks_unfinished_pixels(package, product):
    native = package.native
    # Deep inside the main cardioid at 1e7 (the reference path): every pixel
    # is interior and, with no BLA and no cycle detection, iterates to the
    # 30,000 cap one exact step at a time.
    x, y, zoom, cap = "-0.1", "0.0", b"1e7", 30_000
    handle = native.create_reference(product, x, y, zoom, cap, 256, 3)
    common = dict(disable_bla=1, disable_cycle=1, series_min_terms=32, series_max_terms=32)
    try:
        t0 = time.perf_counter()
        field = native.render_reference(product, handle, 8, 8, zoom, cap, threads=1,
                                        options=native.RenderOptions(time_budget_ms=1, **common))
        elapsed = time.perf_counter() - t0
        unbudgeted = native.render_reference(product, handle, 8, 8, zoom, cap, threads=1,
                                             options=native.RenderOptions(**common))
    finally:
        product.fractal_destroy_reference(handle)
    assert not np.isnan(unbudgeted).any()
    assert (unbudgeted >= cap - 1).all()  # the cell is pathological: all interior
    assert np.isnan(field).any()
    finished = ~np.isnan(field)
    np.testing.assert_array_equal(field[finished], unbudgeted[finished])
    assert elapsed < 5.0, elapsed


@pytest.mark.parametrize("backend", [0, 4])
def test_extreme_zoom_returns_finite_field(package, product, backend):
    native = package.native
    centre = case_defs.centres()["field_e100"]
    handle = native.create_reference(product, centre["re"], centre["im"], b"1e6", 1000, 1024, 3)
    try:
        for zoom in (b"1e100", b"1e4000"):
            field = native.render_reference(product, handle, 8, 8, zoom, 1000,
                                            options=native.RenderOptions(backend=backend))
            assert np.isfinite(field).all(), zoom
    finally:
        product.fractal_destroy_reference(handle)


def test_spill_wait_bound_reports_the_queue_error(package, product, oracle_port):
    native = package.native
    w, h, cap = 320, 180, 5000
    field = torch.empty(w * h, dtype=torch.float32, device="cuda")
    options = native.RenderOptions()
    steps = ctypes.c_ulonglong(0)

    def render():
        status = product.fractal_gb300_render_direct_device(
            ctypes.c_void_p(field.data_ptr()), None, w, h, b"1", b"-0.5", b"0.0", cap, 0, 0.0, 0.0,
            ctypes.byref(options), None)
        assert status == 0, native.last_error(product)

    assert product.fractal_gb300_set_direct_fault_injection(1000, 1) == 0
    try:
        t0 = time.perf_counter()
        render()
        assert product.fractal_gb300_last_direct_steps(ctypes.byref(steps)) == 1
        assert "never published" in native.last_error(product)
        assert time.perf_counter() - t0 < 30.0
    finally:
        assert product.fractal_gb300_set_direct_fault_injection(0, 0) == 0
    # Normal operation again: the same view completes and equals the oracle.
    render()
    assert product.fractal_gb300_last_direct_steps(ctypes.byref(steps)) == 0
    want = native.render_fractal(oracle_port, w, h, b"1", "-0.5", "0.0", cap, 256, False, threads=0)
    np.testing.assert_array_equal(field.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert product.fractal_gb300_set_direct_fault_injection(-1, 0) == 1
