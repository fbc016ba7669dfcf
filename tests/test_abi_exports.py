"""The C-ABI library builds for sm_103a, loads, and exports its header.

CPU-only: no render is attempted except to check that, without a GPU, the
product fails loudly instead of falling back to a CPU path.
"""

from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

from .conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fractal_gb300.h")


def declared_functions() -> list[str]:
    text = open(HEADER, encoding="ascii").read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text)
    keywords = {"if", "sizeof", "defined"}
    return sorted({n for n in names if n not in keywords and (n.startswith("fractal_") or n.startswith("render_"))})


def test_header_declares_the_hot_subset():
    names = declared_functions()
    for required in (
        "fractal_abi_version", "fractal_render_options_version", "fractal_render_options_default",
        "fractal_backend_capabilities", "fractal_last_error", "fractal_set_stats_enabled",
        "fractal_get_last_stats", "fractal_get_last_stats_ex", "fractal_create_reference",
        "fractal_create_reference_reusable", "fractal_create_reference_reusable_options",
        "fractal_create_reference_ex", "fractal_create_reference_ex_options", "fractal_clone_reference",
        "fractal_destroy_reference", "fractal_get_reference_stats", "fractal_render_reference_ex",
        "fractal_render_reference_ex_planes", "fractal_render_mandelbrot_reference_ex",
        "render_mandelbrot_reference", "render_fractal_ex", "render_fractal_ex_planes",
        "render_mandelbrot_ex", "render_mandelbrot", "fractal_colourise",
    ):
        assert required in names


def test_library_exports_every_declared_symbol(product):
    missing = [name for name in declared_functions() if not hasattr(product, name)]
    assert missing == []


def test_abi_version_and_struct_layout(product, package):
    native = package.native
    assert product.fractal_abi_version() == 10
    assert product.fractal_render_options_version() == 2
    assert ctypes.sizeof(native.RenderOptions) == 72
    assert ctypes.sizeof(native.RenderPlanes) == 56
    options = native.RenderOptions()
    options.strict = 7
    product.fractal_render_options_default(ctypes.byref(options))
    assert (options.strict, options.series_min_terms, options.series_max_terms) == (1, 8, 32)
    assert (options.max_bla_length, options.max_linear_bla_length) == (64, 4096)
    assert options.struct_size == 72 and options.version == 2


def test_stats_buffers_validate_capacity(product):
    values = (ctypes.c_uint64 * 39)()
    assert product.fractal_get_last_stats(values, 15) == -1
    assert product.fractal_get_last_stats(values, 16) == 16
    assert product.fractal_get_last_stats_ex(values, 38) == -1
    assert product.fractal_get_last_stats_ex(values, 39) == 39


def test_invalid_handles_are_reported(product):
    values = (ctypes.c_uint64 * 5)()
    assert product.fractal_get_reference_stats(ctypes.c_void_p(0x12345), values, 5) == -1
    assert b"invalid" in product.fractal_last_error()
    product.fractal_destroy_reference(ctypes.c_void_p(0x12345))
    assert b"invalid or already-destroyed" in product.fractal_last_error()
    product.fractal_destroy_reference(None)
    assert product.fractal_last_error() == b""


def test_argument_validation_precedes_device_work(product, package):
    native = package.native
    out = np.empty(4, dtype=np.float32)
    fp = out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    # Zero width, bad formula and bad option versions fail before any GPU use.
    assert product.render_fractal_ex(fp, 0, 2, b"1", b"0", b"0", 100, 256, 0, 0, 0, 0.0, 0.0, None) == 1
    assert b"invalid" in product.fractal_last_error()
    assert product.render_fractal_ex(fp, 2, 2, b"1", b"0", b"0", 100, 256, 0, 0, 9, 0.0, 0.0, None) == 1
    bad = native.RenderOptions()
    bad.version = 1
    assert product.render_fractal_ex(fp, 2, 2, b"1", b"0", b"0", 100, 256, 0, 0, 0, 0.0, 0.0,
                                     ctypes.byref(bad)) == 1
    assert b"unsupported FractalRenderOptions" in product.fractal_last_error()
    opencl = native.RenderOptions(backend=2)
    assert product.render_fractal_ex(fp, 2, 2, b"1", b"0", b"0", 100, 256, 0, 0, 0, 0.0, 0.0,
                                     ctypes.byref(opencl)) == 1
    assert b"OpenCL" in product.fractal_last_error()


def test_no_gpu_means_a_loud_failure(product):
    if product.fractal_gb300_device_count() > 0:
        pytest.skip("a GPU is present; the GPU tests cover rendering")
    out = np.empty(4, dtype=np.float32)
    status = product.render_fractal_ex(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 2, 2, b"1",
                                       b"-0.5", b"0", 100, 256, 0, 0, 0, 0.0, 0.0, None)
    assert status == 1
    assert b"no CUDA device" in product.fractal_last_error()
    assert product.fractal_backend_capabilities() == 0
