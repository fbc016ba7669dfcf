"""ctypes binding of the ``renderer.h`` C ABI (v10) plus the GB300 extensions.

One binding serves every library that exports the ABI: the GB300 library
built from ``csrc/`` (the product), and, in tests only, the CPU oracle
libraries.  The structure mirrors follow the reference loader
(visualizer.py:823-1000 ``NativeRenderOptions`` / ``NativeRenderPlanes``,
visualizer.py:1117-1215 ``NativeKfpOptions``) field for field, because the
ABI is a byte layout contract (renderer.h:43-170).

Errors follow the reference convention: render/colour calls return 0 or 1,
creators return NULL, and the message is read from ``fractal_last_error``
(thread-local in every implementation).  The helpers below turn a failure
into ``RuntimeError`` carrying that message.
"""

from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

ABI_VERSION = 10
RENDER_OPTIONS_VERSION = 2
KFP_OPTIONS_VERSION = 3
KFP_MAX_MULTI_COLORS = 256

FORMULA_IDS = {"mandelbrot": 0, "julia": 1, "burning-ship": 2, "tricorn": 3}

# Capability bits (renderer.h:175-177) plus the CUDA bit this library adds.
# The reference loader tests ``1 << backend`` (visualizer.py:1286); backend
# id 4 therefore maps to bit 16 and does not alias the OpenCL GPU bit 8.
CAPABILITY_SCALAR = 1
CAPABILITY_AVX2 = 2
CAPABILITY_OPENCL = 4
CAPABILITY_OPENCL_GPU = 8
BACKEND_CUDA = 4
CAPABILITY_CUDA = 1 << BACKEND_CUDA

STATS_FIELDS = (
    "pixels",
    "logical_iterations",
    "bla_blocks",
    "linear_blocks",
    "cubic_blocks",
    "exact_steps",
    "replay_steps",
    "bla_retries",
    "cycle_inside",
    "double_tail_pixels",
    "bla_disabled_pixels",
    "tail_steps",
    "max_tail_steps",
    "tail_rebases",
    "tail_rebase_fallbacks",
    "max_pixel_iterations",
)
EXTENDED_STATS_FIELDS = STATS_FIELDS + (
    "series_pixels",
    "series_jumps",
    "glitch_count",
    "unresolved_pixels",
    "deadline_aborts",
    "secondary_references",
    "render_ns",
) + tuple(f"bla_length_bin_{index}" for index in range(16))


class RenderOptions(ctypes.Structure):
    """``FractalRenderOptions`` (renderer.h:43-67)."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("version", ctypes.c_uint32),
        ("strict", ctypes.c_int32),
        ("allow_recovery", ctypes.c_int32),
        ("time_budget_ms", ctypes.c_int32),
        ("disable_bla", ctypes.c_int32),
        ("disable_cycle", ctypes.c_int32),
        ("strict_cycle", ctypes.c_int32),
        ("series_min_terms", ctypes.c_int32),
        ("series_max_terms", ctypes.c_int32),
        ("max_bla_length", ctypes.c_int32),
        ("max_linear_bla_length", ctypes.c_int32),
        ("backend", ctypes.c_int32),
        ("escape_radius_mode", ctypes.c_int32),
        ("coordinate_mode", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 1),
        ("output_bias", ctypes.c_double),
    ]

    def __init__(self, **values) -> None:
        super().__init__()
        # The library default (renderer.cpp:4708-4727) is the starting point.
        self.struct_size = ctypes.sizeof(self)
        self.version = RENDER_OPTIONS_VERSION
        self.strict = 1
        self.allow_recovery = 0
        self.time_budget_ms = 0
        self.disable_bla = 0
        self.disable_cycle = 0
        self.strict_cycle = 0
        self.series_min_terms = 8
        self.series_max_terms = 32
        self.max_bla_length = 64
        self.max_linear_bla_length = 4096
        self.backend = 0
        self.escape_radius_mode = 0
        self.coordinate_mode = 0
        self.output_bias = 0.0
        for key, value in values.items():
            if key == "plane_flags":
                self.reserved[0] = int(value)
            else:
                setattr(self, key, value)


class RenderPlanes(ctypes.Structure):
    """``FractalRenderPlanes`` (renderer.h:155-170)."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("version", ctypes.c_uint32),
        ("orbit_iteration", ctypes.POINTER(ctypes.c_int64)),
        ("phase", ctypes.POINTER(ctypes.c_double)),
        ("de_x", ctypes.POINTER(ctypes.c_double)),
        ("de_y", ctypes.POINTER(ctypes.c_double)),
        ("test1", ctypes.POINTER(ctypes.c_double)),
        ("test2", ctypes.POINTER(ctypes.c_double)),
    ]


class KfpPlanes(ctypes.Structure):
    """``FractalKfpPlanes`` (renderer.h:135-153)."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("version", ctypes.c_uint32),
        ("orbit_iteration", ctypes.POINTER(ctypes.c_int64)),
        ("bailout", ctypes.POINTER(ctypes.c_double)),
        ("iteration", ctypes.POINTER(ctypes.c_int64)),
        ("transition", ctypes.POINTER(ctypes.c_double)),
        ("phase", ctypes.POINTER(ctypes.c_double)),
        ("de_x", ctypes.POINTER(ctypes.c_double)),
        ("de_y", ctypes.POINTER(ctypes.c_double)),
        ("test1", ctypes.POINTER(ctypes.c_double)),
        ("test2", ctypes.POINTER(ctypes.c_double)),
        ("texture_rgb", ctypes.POINTER(ctypes.c_uint8)),
        ("texture_width", ctypes.c_int32),
        ("texture_height", ctypes.c_int32),
        ("texture_stride", ctypes.c_int32),
    ]


class KfpOptions(ctypes.Structure):
    """``FractalKfpOptions`` version 3 (renderer.h:75-119)."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("version", ctypes.c_uint32),
        ("iter_div", ctypes.c_double),
        ("color_offset", ctypes.c_double),
        ("ratio", ctypes.c_double),
        ("color_method", ctypes.c_int32),
        ("smooth_method", ctypes.c_int32),
        ("smooth", ctypes.c_int32),
        ("flat", ctypes.c_int32),
        ("inverse_transition", ctypes.c_int32),
        ("phase_color_strength", ctypes.c_double),
        ("multi_color", ctypes.c_int32),
        ("blend_multi_color", ctypes.c_int32),
        ("multi_color_count", ctypes.c_uint32),
        ("multi_color_period", ctypes.c_double * KFP_MAX_MULTI_COLORS),
        ("multi_color_start", ctypes.c_int32 * KFP_MAX_MULTI_COLORS),
        ("multi_color_type", ctypes.c_int32 * KFP_MAX_MULTI_COLORS),
        ("power", ctypes.c_double),
        ("slopes", ctypes.c_int32),
        ("slope_power", ctypes.c_double),
        ("slope_ratio", ctypes.c_double),
        ("slope_angle", ctypes.c_double),
        ("differences", ctypes.c_int32),
        ("interior_color", ctypes.c_int32 * 3),
        ("field_bias", ctypes.c_double),
        ("bailout_radius_preset", ctypes.c_int32),
        ("bailout_radius_custom", ctypes.c_double),
        ("bailout_norm_preset", ctypes.c_int32),
        ("bailout_norm_custom", ctypes.c_double),
        ("texture_enabled", ctypes.c_int32),
        ("texture_merge", ctypes.c_double),
        ("texture_power", ctypes.c_double),
        ("texture_ratio", ctypes.c_double),
        ("texture_resize", ctypes.c_int32),
        ("use_opengl", ctypes.c_int32),
        ("use_srgb", ctypes.c_int32),
        ("show_glitches", ctypes.c_int32),
    ]


_c_float_p = ctypes.POINTER(ctypes.c_float)
_c_u8_p = ctypes.POINTER(ctypes.c_uint8)
_c_u32_p = ctypes.POINTER(ctypes.c_uint32)
_c_u64_p = ctypes.POINTER(ctypes.c_uint64)
_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_i32_p = ctypes.POINTER(ctypes.c_int32)

# (name, restype, argtypes) for the renderer.h hot subset.
_ABI = (
    ("fractal_abi_version", ctypes.c_int, ()),
    ("fractal_render_options_version", ctypes.c_int, ()),
    ("fractal_render_options_default", None, (ctypes.POINTER(RenderOptions),)),
    ("fractal_backend_capabilities", ctypes.c_int, ()),
    ("fractal_last_error", ctypes.c_char_p, ()),
    ("fractal_set_stats_enabled", None, (ctypes.c_int,)),
    ("fractal_get_last_stats", ctypes.c_int, (_c_u64_p, ctypes.c_int)),
    ("fractal_get_last_stats_ex", ctypes.c_int, (_c_u64_p, ctypes.c_int)),
    ("fractal_create_reference", ctypes.c_void_p,
     (ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int)),
    ("fractal_create_reference_reusable", ctypes.c_void_p,
     (ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int)),
    ("fractal_create_reference_reusable_options", ctypes.c_void_p,
     (ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.POINTER(RenderOptions))),
    ("fractal_create_reference_ex", ctypes.c_void_p,
     (ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p)),
    ("fractal_create_reference_ex_options", ctypes.c_void_p,
     (ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
      ctypes.POINTER(RenderOptions))),
    ("fractal_clone_reference", ctypes.c_void_p, (ctypes.c_void_p, ctypes.c_char_p)),
    ("fractal_destroy_reference", None, (ctypes.c_void_p,)),
    ("fractal_get_reference_stats", ctypes.c_int,
     (ctypes.c_void_p, _c_u64_p, ctypes.c_int)),
    ("fractal_render_reference_ex", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p,
      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(RenderOptions))),
    ("fractal_render_mandelbrot_reference_ex", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p,
      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(RenderOptions))),
    ("fractal_render_reference_ex_planes", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p,
      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(RenderOptions), ctypes.POINTER(RenderPlanes))),
    ("render_mandelbrot_reference", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_void_p,
      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int)),
    ("render_fractal_ex", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
      ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.POINTER(RenderOptions))),
    ("render_fractal_ex_planes", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
      ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.POINTER(RenderOptions),
      ctypes.POINTER(RenderPlanes))),
    ("render_mandelbrot_ex", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
      ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(RenderOptions))),
    ("render_mandelbrot", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
      ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int)),
    ("fractal_colourise", ctypes.c_int,
     (_c_float_p, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int)),
    ("fractal_colourise_kfp", ctypes.c_int,
     (_c_float_p, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(KfpOptions),
      _c_u8_p, ctypes.c_int, ctypes.c_int)),
    ("fractal_atlas_colourise_kfp", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int,
      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.POINTER(KfpOptions), _c_u8_p, ctypes.c_int, ctypes.c_int)),
    ("fractal_atlas_colourise_kfp_planes", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(KfpPlanes), _c_float_p, ctypes.c_int,
      ctypes.c_int, ctypes.c_int, ctypes.POINTER(KfpPlanes), _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.POINTER(KfpOptions), _c_u8_p, ctypes.c_int, ctypes.c_int)),
    ("fractal_colourise_kfp_planes", ctypes.c_int,
     (_c_float_p, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(KfpOptions),
      ctypes.POINTER(KfpPlanes), _c_u8_p, ctypes.c_int, ctypes.c_int)),
    ("fractal_colourise_kfp_precise", ctypes.c_int,
     (_c_float_p, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(KfpOptions),
      _c_u8_p, ctypes.c_int, ctypes.c_int)),
    ("fractal_colourise_accents", ctypes.c_int,
     (_c_float_p, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, _c_u8_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_int)),
    ("fractal_atlas_colourise_kfp_raw", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
      ctypes.POINTER(KfpOptions), _c_u8_p, ctypes.c_int, ctypes.c_int)),
    ("fractal_atlas_colourise_kfp_raw_precise", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
      ctypes.POINTER(KfpOptions), _c_u8_p, ctypes.c_int, ctypes.c_int)),
    ("fractal_render_points", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_char_p, _c_double_p, _c_double_p, ctypes.POINTER(ctypes.c_int32),
      ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(RenderOptions))),
    ("fractal_render_points_ex_planes", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_char_p, _c_double_p, _c_double_p, ctypes.POINTER(ctypes.c_int32),
      ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(RenderOptions),
      ctypes.POINTER(RenderPlanes))),
    ("fractal_crop_field", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_int)),
    ("fractal_crop_rgb", ctypes.c_int,
     (_c_u8_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int)),
    ("fractal_atlas_composite_rgb", ctypes.c_int,
     (_c_u8_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int,
      ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int)),
    ("fractal_crop_colourise", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int)),
    ("fractal_crop_colourise_interior", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_int)),
    ("fractal_crop_colourise_accents", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _c_u8_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_int)),
    ("fractal_crop_colourise_kfp", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(KfpOptions), _c_u8_p,
      ctypes.c_int, ctypes.c_int)),
    ("fractal_crop_colourise_kfp_precise", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(KfpOptions), _c_u8_p,
      ctypes.c_int, ctypes.c_int)),
    # Atlas compositor (renderer.h:797-836, 997-1067).
    ("fractal_atlas_field", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
      ctypes.c_int)),
    ("fractal_atlas_field_ex", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
      ctypes.c_int)),
    ("fractal_atlas_colourise", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int)),
    ("fractal_atlas_colourise_interior", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_int)),
    ("fractal_atlas_colourise_accents", ctypes.c_int,
     (_c_float_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_float_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, _c_u8_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _c_u8_p, ctypes.c_int,
      ctypes.c_int, ctypes.c_int, ctypes.c_int)),
)

# GB300 extensions (include/fractal_gb300.h).  Absent from the CPU oracles.
class Keyframe(ctypes.Structure):
    """FractalGb300Keyframe: one frame of a batched device render."""

    _fields_ = [
        ("field", ctypes.c_void_p),
        ("counts", ctypes.c_void_p),
        ("zoom_text", ctypes.c_char_p),
        ("reference", ctypes.c_void_p),
        ("max_iter", ctypes.c_int),
        ("flags", ctypes.c_int),
    ]


class Field(ctypes.Structure):
    """FractalGb300Field: one field of a general batched device render."""

    _fields_ = [
        ("field", ctypes.c_void_p),
        ("counts", ctypes.c_void_p),
        ("de_x", ctypes.c_void_p),
        ("de_y", ctypes.c_void_p),
        ("zoom_text", ctypes.c_char_p),
        ("reference", ctypes.c_void_p),
        ("width", ctypes.c_int),
        ("height", ctypes.c_int),
        ("max_iter", ctypes.c_int),
        ("flags", ctypes.c_int),
    ]


BATCH_GRAPH = 1
BATCH_AUTOTUNE = 2
BATCH_TILES = 4
BATCH_LEARNED = 8
BATCH_PROBE = 16
BATCH_FP32_ALTERNATES = 32
KEYFRAME_SHALLOW = 1

_GB300_ABI = (
    ("fractal_gb300_device_count", ctypes.c_int, ()),
    ("fractal_gb300_set_table_builder", None, (ctypes.c_int,)),
    ("fractal_gb300_last_kernel_ms", ctypes.c_double, ()),
    ("fractal_gb300_check_division", ctypes.c_int, (ctypes.c_float, ctypes.POINTER(ctypes.c_ulonglong))),
    ("fractal_gb300_render_reference_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
      ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(RenderOptions), ctypes.c_int, ctypes.c_void_p)),
    ("fractal_gb300_render_direct_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
      ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
      ctypes.c_double, ctypes.POINTER(RenderOptions), ctypes.c_void_p)),
    ("fractal_gb300_fma_peak", ctypes.c_int, (ctypes.c_int, ctypes.POINTER(ctypes.c_double))),
    ("fractal_gb300_colourise_kfp_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(KfpOptions), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p)),
    ("fractal_gb300_colourise_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
      ctypes.c_void_p)),
    ("fractal_gb300_atlas_field_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
      ctypes.c_void_p)),
    ("fractal_gb300_atlas_colourise_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_int),
      _c_u8_p, ctypes.c_void_p)),
    ("fractal_gb300_atlas_colourise_kfp_raw_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
      ctypes.c_double, ctypes.c_int, ctypes.POINTER(KfpOptions), ctypes.c_void_p, ctypes.c_int,
      ctypes.c_void_p)),
    ("fractal_gb300_atlas_kfp_surface_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
      ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
      ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_void_p)),
    ("fractal_gb300_atlas_last_exact_pixels", ctypes.c_longlong, ()),
    ("fractal_gb300_packed_frame_bytes", ctypes.c_longlong, (ctypes.c_int, ctypes.c_int, ctypes.c_int)),
    ("fractal_gb300_pack_frame_device", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)),
    ("fractal_gb300_render_keyframes_device", ctypes.c_int,
     (ctypes.POINTER(Keyframe), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
      ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(RenderOptions), ctypes.c_int,
      ctypes.c_uint, ctypes.c_void_p)),
    ("fractal_gb300_render_fields_device", ctypes.c_int,
     (ctypes.POINTER(Field), ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
      ctypes.POINTER(RenderOptions), ctypes.c_int, ctypes.c_uint, ctypes.c_void_p)),
    ("fractal_gb300_queue_shapes", ctypes.c_int, (ctypes.POINTER(ctypes.c_int), ctypes.c_int)),
    ("fractal_gb300_set_direct_fault_injection", ctypes.c_int, (ctypes.c_int, ctypes.c_int)),
    ("fractal_gb300_set_queue_shapes", ctypes.c_int, (ctypes.POINTER(ctypes.c_int), ctypes.c_int)),
    ("fractal_gb300_set_cost_network", ctypes.c_int, (ctypes.c_void_p,)),
    ("fractal_gb300_last_direct_steps", ctypes.c_int, (ctypes.POINTER(ctypes.c_ulonglong),)),
    ("fractal_gb300_last_tiles", ctypes.c_int,
     (ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
      ctypes.POINTER(ctypes.c_double))),
    ("fractal_gb300_costnet_create", ctypes.c_void_p, (ctypes.c_uint,)),
    ("fractal_gb300_costnet_destroy", None, (ctypes.c_void_p,)),
    ("fractal_gb300_costnet_parameter_count", ctypes.c_int, ()),
    ("fractal_gb300_costnet_parameters", ctypes.c_int,
     (ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_int)),
    ("fractal_gb300_costnet_train_step", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_int,
      ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_void_p)),
    ("fractal_gb300_costnet_predict", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)),
    ("fractal_gb300_gemm_bf16", ctypes.c_int,
     (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
      ctypes.c_void_p)),
)


class NativeError(RuntimeError):
    """A library call reported failure; the message is fractal_last_error()."""


def _bind(library: ctypes.CDLL, table, required: bool) -> None:
    for name, restype, argtypes in table:
        function = getattr(library, name, None)
        if function is None:
            if required:
                raise NativeError(f"{library._name} does not export {name}")
            continue
        function.restype = restype
        function.argtypes = list(argtypes)


def load(path: str, *, gb300: bool = False) -> ctypes.CDLL:
    """Load and type one ABI v10 library, rejecting other ABI versions.

    The version gate mirrors the reference loader (visualizer.py:1550).
    """
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    library = ctypes.CDLL(os.path.abspath(path))
    _bind(library, _ABI, required=False)
    _bind(library, _GB300_ABI, required=gb300)
    version = library.fractal_abi_version()
    if version != ABI_VERSION:
        raise NativeError(f"{path}: ABI version {version}, expected {ABI_VERSION}")
    return library


def last_error(library: ctypes.CDLL) -> str:
    message = library.fractal_last_error()
    return (message or b"").decode("utf-8", errors="replace")


def _check(library: ctypes.CDLL, status: int, what: str) -> None:
    if status != 0:
        raise NativeError(f"{what} failed: {last_error(library)}")


def _text(value) -> bytes:
    return value if isinstance(value, bytes) else str(value).encode("ascii")


def zoom_text(log10_zoom: float) -> bytes:
    """Decimal zoom string used by the reference pipeline (visualizer.py:5118-5124)."""
    import math

    exponent = math.floor(log10_zoom)
    mantissa = 10.0 ** (log10_zoom - exponent)
    return f"{mantissa:.17g}e{exponent:+d}".encode("ascii")


def create_reference(
    library: ctypes.CDLL,
    x_center: str,
    y_center: str,
    zoom: bytes,
    max_iter: int,
    precision_bits: int,
    series_order: int = 32,
    *,
    formula: str = "mandelbrot",
    julia: tuple[str, str] = ("0", "0"),
    options: Optional[RenderOptions] = None,
    reusable: bool = False,
) -> int:
    """Create a reference handle through the same creators the reference uses."""
    formula_id = FORMULA_IDS[formula]
    if formula_id == 0 and options is not None:
        # Option-aware Mandelbrot roots are always reusable
        # (visualizer.py:6330-6346).
        handle = library.fractal_create_reference_reusable_options(
            _text(x_center), _text(y_center), _text(zoom), max_iter, precision_bits,
            series_order, ctypes.byref(options))
    elif formula_id != 0:
        handle = library.fractal_create_reference_ex_options(
            _text(x_center), _text(y_center), _text(zoom), max_iter, precision_bits,
            series_order, formula_id, _text(julia[0]), _text(julia[1]),
            ctypes.byref(options) if options is not None else None)
    elif reusable:
        handle = library.fractal_create_reference_reusable(
            _text(x_center), _text(y_center), _text(zoom), max_iter, precision_bits,
            series_order)
    else:
        handle = library.fractal_create_reference(
            _text(x_center), _text(y_center), _text(zoom), max_iter, precision_bits,
            series_order)
    if not handle:
        raise NativeError(f"reference creation failed: {last_error(library)}")
    return handle


def clone_reference(library: ctypes.CDLL, handle: int, zoom: bytes) -> int:
    clone = library.fractal_clone_reference(handle, _text(zoom))
    if not clone:
        raise NativeError(f"reference clone failed: {last_error(library)}")
    return clone


def allocate_planes(width: int, height: int):
    """Allocate the six render planes; returns (struct, dict of numpy arrays)."""
    count = width * height
    arrays = {
        "orbit_iteration": np.zeros(count, dtype=np.int64),
        "phase": np.zeros(count, dtype=np.float64),
        "de_x": np.zeros(count, dtype=np.float64),
        "de_y": np.zeros(count, dtype=np.float64),
        "test1": np.zeros(count, dtype=np.float64),
        "test2": np.zeros(count, dtype=np.float64),
    }
    planes = RenderPlanes()
    planes.struct_size = ctypes.sizeof(RenderPlanes)
    planes.version = 1
    planes.orbit_iteration = arrays["orbit_iteration"].ctypes.data_as(
        ctypes.POINTER(ctypes.c_int64))
    for key in ("phase", "de_x", "de_y", "test1", "test2"):
        setattr(planes, key, arrays[key].ctypes.data_as(_c_double_p))
    return planes, arrays


def render_reference(
    library: ctypes.CDLL,
    handle: int,
    width: int,
    height: int,
    zoom: bytes,
    max_iter: int,
    *,
    threads: int = 0,
    series_order: int = 3,
    series_block: int = 256,
    options: Optional[RenderOptions] = None,
    planes: bool = False,
):
    """Render one field from a prepared reference.

    Returns the float32 field, and with ``planes=True`` also the plane arrays.
    """
    output = np.empty(width * height, dtype=np.float32)
    options = options or RenderOptions()
    if planes:
        plane_struct, arrays = allocate_planes(width, height)
        status = library.fractal_render_reference_ex_planes(
            output.ctypes.data_as(_c_float_p), width, height, _text(zoom), handle,
            max_iter, threads, series_order, series_block, ctypes.byref(options),
            ctypes.byref(plane_struct))
        _check(library, status, "fractal_render_reference_ex_planes")
        return output, arrays
    status = library.fractal_render_reference_ex(
        output.ctypes.data_as(_c_float_p), width, height, _text(zoom), handle, max_iter,
        threads, series_order, series_block, ctypes.byref(options))
    _check(library, status, "fractal_render_reference_ex")
    return output


def render_fractal(
    library: ctypes.CDLL,
    width: int,
    height: int,
    zoom: bytes,
    x_center: str,
    y_center: str,
    max_iter: int,
    precision_bits: int,
    use_perturbation: bool,
    *,
    threads: int = 0,
    formula: str = "mandelbrot",
    julia: tuple[float, float] = (0.0, 0.0),
    options: Optional[RenderOptions] = None,
    planes: bool = False,
):
    """``render_fractal_ex[_planes]``: one-shot field render (renderer.h:323-360)."""
    output = np.empty(width * height, dtype=np.float32)
    options = options or RenderOptions()
    arguments = (
        output.ctypes.data_as(_c_float_p), width, height, _text(zoom), _text(x_center),
        _text(y_center), max_iter, precision_bits, int(use_perturbation), threads,
        FORMULA_IDS[formula], float(julia[0]), float(julia[1]), ctypes.byref(options))
    if planes:
        plane_struct, arrays = allocate_planes(width, height)
        status = library.render_fractal_ex_planes(*arguments, ctypes.byref(plane_struct))
        _check(library, status, "render_fractal_ex_planes")
        return output, arrays
    status = library.render_fractal_ex(*arguments)
    _check(library, status, "render_fractal_ex")
    return output


def colourise(
    library: ctypes.CDLL,
    field: np.ndarray,
    width: int,
    height: int,
    max_iter: int,
    phase: float,
    vocal: float,
    instrumental: float,
    pitch: float,
    threads: int = 0,
) -> np.ndarray:
    """``fractal_colourise`` (aurora palette, renderer.h:400-411)."""
    field = np.ascontiguousarray(field, dtype=np.float32)
    output = np.empty(width * height * 3, dtype=np.uint8)
    status = library.fractal_colourise(
        field.ctypes.data_as(_c_float_p), output.ctypes.data_as(_c_u8_p), width, height,
        max_iter, phase, vocal, instrumental, pitch, threads)
    _check(library, status, "fractal_colourise")
    return output


def _float_in(array):
    if array is None:
        return None
    return np.ascontiguousarray(array, dtype=np.float32)


def atlas_field(library, parent, parent_shape, parent_max_iter, child, child_shape, child_max_iter,
                output_shape, parent_zoom, child_fraction, palette_max_iter, *, child_zoom=None,
                parent_bias=None, child_bias=None, output_bias=None, feather=None, threads=0) -> np.ndarray:
    """Scalar atlas frame: ``fractal_atlas_field_ex`` (renderer.h:815-836)
    when any extended argument is given, else ``fractal_atlas_field``.
    Shapes are (width, height)."""
    parent, child = _float_in(parent), _float_in(child)
    width, height = output_shape
    output = np.empty(width * height, dtype=np.float32)
    child_ptr = child.ctypes.data_as(_c_float_p) if child is not None else None
    cw, ch = child_shape if child_shape else (0, 0)
    extended = any(v is not None for v in (child_zoom, parent_bias, child_bias, output_bias, feather))
    if extended:
        status = library.fractal_atlas_field_ex(
            parent.ctypes.data_as(_c_float_p), parent_shape[0], parent_shape[1], parent_max_iter, child_ptr, cw,
            ch, child_max_iter, output.ctypes.data_as(_c_float_p), width, height, parent_zoom, child_fraction,
            1.0 if child_zoom is None else child_zoom, parent_bias or 0.0, child_bias or 0.0, output_bias or 0.0,
            palette_max_iter, 48 if feather is None else feather, threads)
    else:
        status = library.fractal_atlas_field(
            parent.ctypes.data_as(_c_float_p), parent_shape[0], parent_shape[1], parent_max_iter, child_ptr, cw,
            ch, child_max_iter, output.ctypes.data_as(_c_float_p), width, height, parent_zoom, child_fraction,
            palette_max_iter, threads)
    _check(library, status, "fractal_atlas_field")
    return output


def atlas_colourise(library, parent, parent_shape, parent_max_iter, child, child_shape, child_max_iter,
                    output_shape, parent_zoom, child_fraction, palette_max_iter, phase, vocal, instrumental,
                    pitch, *, interior=None, accents=None, threads=0) -> np.ndarray:
    """Aurora atlas frame (renderer.h:997-1067): ``fractal_atlas_colourise``,
    ``_interior`` (interior RGB given) or ``_accents`` (accents given)."""
    parent, child = _float_in(parent), _float_in(child)
    width, height = output_shape
    output = np.empty(width * height * 3, dtype=np.uint8)
    child_ptr = child.ctypes.data_as(_c_float_p) if child is not None else None
    cw, ch = child_shape if child_shape else (0, 0)
    common = (parent.ctypes.data_as(_c_float_p), parent_shape[0], parent_shape[1], parent_max_iter, child_ptr, cw,
              ch, child_max_iter, output.ctypes.data_as(_c_u8_p), width, height, parent_zoom, child_fraction,
              palette_max_iter, phase, vocal, instrumental, pitch)
    if accents is not None:
        accents = np.ascontiguousarray(accents, dtype=np.uint8).reshape(9)
        red, green, blue = interior if interior is not None else (0, 0, 0)
        status = library.fractal_atlas_colourise_accents(*common, accents.ctypes.data_as(_c_u8_p), red, green,
                                                         blue, threads)
    elif interior is not None:
        status = library.fractal_atlas_colourise_interior(*common, *interior, threads)
    else:
        status = library.fractal_atlas_colourise(*common, threads)
    _check(library, status, "fractal_atlas_colourise")
    return output


def atlas_colourise_kfp_raw(library, parent, parent_shape, parent_max_iter, child, child_shape, child_max_iter,
                            output_shape, parent_zoom, child_fraction, child_zoom, max_iter, options, lut,
                            colour=(0.0, 0.0, 0.0, 0.5), threads=0) -> np.ndarray:
    """``fractal_atlas_colourise_kfp_raw`` (renderer.h:663-687): parent and
    child composed into one scalar surface, then one KFP pass.  `options` is
    a KfpOptions block, `lut` the N x 3 palette."""
    parent, child = _float_in(parent), _float_in(child)
    lut = np.ascontiguousarray(lut, dtype=np.uint8)
    width, height = output_shape
    output = np.empty(width * height * 3, dtype=np.uint8)
    child_ptr = child.ctypes.data_as(_c_float_p) if child is not None else None
    cw, ch = child_shape if child_shape else (0, 0)
    status = library.fractal_atlas_colourise_kfp_raw(
        parent.ctypes.data_as(_c_float_p), parent_shape[0], parent_shape[1], parent_max_iter, child_ptr, cw, ch,
        child_max_iter, output.ctypes.data_as(_c_u8_p), width, height, parent_zoom, child_fraction, child_zoom,
        max_iter, *colour, ctypes.byref(options), lut.ctypes.data_as(_c_u8_p), lut.shape[0], threads)
    _check(library, status, "fractal_atlas_colourise_kfp_raw")
    return output


def render_points(library, handle: int, zoom: bytes, real, imag, exponents, max_iter: int, *, threads: int = 0,
                  series_order: int = 3, series_block: int = 256, options: Optional[RenderOptions] = None,
                  planes: bool = False):
    """``fractal_render_points[_ex_planes]`` (renderer.h:287-320): one value
    per offset (real * 2^e, imag * 2^e) from the reference centre; returns
    (field, planes dict or None)."""
    real = np.ascontiguousarray(real, dtype=np.float64)
    imag = np.ascontiguousarray(imag, dtype=np.float64)
    exponents = np.ascontiguousarray(exponents, dtype=np.int32)
    count = real.size
    field = np.empty(count, dtype=np.float32)
    options = options or RenderOptions()
    args = (field.ctypes.data_as(_c_float_p), count, _text(zoom), real.ctypes.data_as(_c_double_p),
            imag.ctypes.data_as(_c_double_p), exponents.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), handle,
            max_iter, threads, series_order, series_block, ctypes.byref(options))
    if planes:
        plane_struct, arrays = allocate_planes(count, 1)
        status = library.fractal_render_points_ex_planes(*args, ctypes.byref(plane_struct))
        _check(library, status, "fractal_render_points_ex_planes")
        return field, arrays
    status = library.fractal_render_points(*args)
    _check(library, status, "fractal_render_points")
    return field, None


def kfp_planes_struct(planes: dict):
    """A FractalKfpPlanes over the arrays of `planes` (field names; absent
    names pass NULL; ``texture`` = (top-down RGB8 rows, width, height,
    stride)); returns (struct, arrays to keep alive)."""
    struct = KfpPlanes()
    struct.struct_size = ctypes.sizeof(KfpPlanes)
    struct.version = 1
    keep = []
    for name in ("orbit_iteration", "iteration"):
        if planes.get(name) is not None:
            array = np.ascontiguousarray(planes[name], dtype=np.int64)
            keep.append(array)
            setattr(struct, name, array.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    for name in ("bailout", "transition", "phase", "de_x", "de_y", "test1", "test2"):
        if planes.get(name) is not None:
            array = np.ascontiguousarray(planes[name], dtype=np.float64)
            keep.append(array)
            setattr(struct, name, array.ctypes.data_as(_c_double_p))
    if planes.get("texture") is not None:
        rows, struct.texture_width, struct.texture_height, struct.texture_stride = planes["texture"]
        rows = np.ascontiguousarray(rows, dtype=np.uint8)
        keep.append(rows)
        struct.texture_rgb = rows.ctypes.data_as(_c_u8_p)
    return struct, keep


def atlas_colourise_kfp(library, parent, output_shape, child, child_shape, child_origin, feather, max_iter, options,
                        lut, colour=(0.0, 0.0, 0.0, 0.5), threads: int = 0) -> np.ndarray:
    """``fractal_atlas_colourise_kfp`` (renderer.h:554-576): separate KFP
    tiles, the output-sized parent and a child rectangle at `child_origin`."""
    width, height = output_shape
    parent = np.ascontiguousarray(parent, dtype=np.float32)
    lut = np.ascontiguousarray(lut, dtype=np.uint8)
    cw, ch = child_shape if child is not None else (0, 0)
    left, top = child_origin if child is not None else (0, 0)
    child_ptr = None
    if child is not None:
        child = np.ascontiguousarray(child, dtype=np.float32)
        child_ptr = child.ctypes.data_as(_c_float_p)
    output = np.empty(width * height * 3, dtype=np.uint8)
    status = library.fractal_atlas_colourise_kfp(
        parent.ctypes.data_as(_c_float_p), width, height, child_ptr, cw, ch, output.ctypes.data_as(_c_u8_p), width,
        height, max_iter, left, top, feather if child is not None else 0, *colour, ctypes.byref(options),
        lut.ctypes.data_as(_c_u8_p), lut.shape[0], threads)
    _check(library, status, "fractal_atlas_colourise_kfp")
    return output


def atlas_colourise_kfp_planes(library, parent, parent_shape, parent_max_iter, parent_planes, child, child_shape,
                               child_max_iter, child_planes, output_shape, parent_zoom, child_fraction, child_zoom,
                               max_iter, centered_input, options, lut, colour=(0.0, 0.0, 0.0, 0.5),
                               threads: int = 0) -> np.ndarray:
    """``fractal_atlas_colourise_kfp_planes`` (renderer.h:604-631); plane
    dicts as for :func:`kfp_planes_struct` (None: no child)."""
    width, height = output_shape
    parent = np.ascontiguousarray(parent, dtype=np.float32)
    lut = np.ascontiguousarray(lut, dtype=np.uint8)
    parent_struct, keep = kfp_planes_struct(parent_planes)
    child_ptr = child_struct_ref = None
    cw, ch = child_shape if child is not None else (0, 0)
    if child is not None:
        child = np.ascontiguousarray(child, dtype=np.float32)
        child_ptr = child.ctypes.data_as(_c_float_p)
        child_struct, more = kfp_planes_struct(child_planes)
        keep += more
        child_struct_ref = ctypes.byref(child_struct)
    output = np.empty(width * height * 3, dtype=np.uint8)
    status = library.fractal_atlas_colourise_kfp_planes(
        parent.ctypes.data_as(_c_float_p), parent_shape[0], parent_shape[1], parent_max_iter,
        ctypes.byref(parent_struct), child_ptr, cw, ch, child_max_iter if child is not None else 0, child_struct_ref,
        output.ctypes.data_as(_c_u8_p), width, height, parent_zoom, child_fraction, child_zoom, max_iter,
        centered_input, *colour, ctypes.byref(options), lut.ctypes.data_as(_c_u8_p), lut.shape[0], threads)
    _check(library, status, "fractal_atlas_colourise_kfp_planes")
    return output


def colourise_kfp_planes(library, field, width: int, height: int, max_iter: int, options, planes: dict, lut,
                         colour=(0.0, 0.0, 0.0, 0.5), threads: int = 0) -> np.ndarray:
    """``fractal_colourise_kfp_planes`` (renderer.h:483-497); `planes` maps
    FractalKfpPlanes field names to arrays (absent names pass NULL), and
    ``texture`` to (top-down RGB8 rows, width, height, stride)."""
    field = np.ascontiguousarray(field, dtype=np.float32)
    lut = np.ascontiguousarray(lut, dtype=np.uint8)
    struct, keep = kfp_planes_struct(planes)
    output = np.empty(width * height * 3, dtype=np.uint8)
    status = library.fractal_colourise_kfp_planes(
        field.ctypes.data_as(_c_float_p), output.ctypes.data_as(_c_u8_p), width, height, max_iter, *colour,
        ctypes.byref(options), ctypes.byref(struct), lut.ctypes.data_as(_c_u8_p), lut.shape[0], threads)
    _check(library, status, "fractal_colourise_kfp_planes")
    return output


def crop_field(library, source, source_shape, output_shape, zoom, threads=0) -> np.ndarray:
    """``fractal_crop_field`` (renderer.h:786-795): plain bilinear crop."""
    source = np.ascontiguousarray(source, dtype=np.float32)
    width, height = output_shape
    output = np.empty(width * height, dtype=np.float32)
    status = library.fractal_crop_field(source.ctypes.data_as(_c_float_p), source_shape[0], source_shape[1],
                                        output.ctypes.data_as(_c_float_p), width, height, zoom, threads)
    _check(library, status, "fractal_crop_field")
    return output


def crop_rgb(library, source, source_shape, output_shape, zoom, threads=0) -> np.ndarray:
    """``fractal_crop_rgb`` (renderer.h:716-725)."""
    source = np.ascontiguousarray(source, dtype=np.uint8)
    width, height = output_shape
    output = np.empty(width * height * 3, dtype=np.uint8)
    status = library.fractal_crop_rgb(source.ctypes.data_as(_c_u8_p), source_shape[0], source_shape[1],
                                      output.ctypes.data_as(_c_u8_p), width, height, zoom, threads)
    _check(library, status, "fractal_crop_rgb")
    return output


def atlas_composite_rgb(library, parent, parent_shape, child, child_shape, output_shape, parent_zoom,
                        child_fraction, child_zoom, feather, threads=0) -> np.ndarray:
    """``fractal_atlas_composite_rgb`` (renderer.h:726-741): coloured parent
    and child tiles composed with a smoothstep seam."""
    parent = np.ascontiguousarray(parent, dtype=np.uint8)
    child = None if child is None else np.ascontiguousarray(child, dtype=np.uint8)
    width, height = output_shape
    output = np.empty(width * height * 3, dtype=np.uint8)
    cw, ch = child_shape if child is not None else (0, 0)
    status = library.fractal_atlas_composite_rgb(
        parent.ctypes.data_as(_c_u8_p), parent_shape[0], parent_shape[1],
        child.ctypes.data_as(_c_u8_p) if child is not None else None, cw, ch, output.ctypes.data_as(_c_u8_p),
        width, height, parent_zoom, child_fraction, child_zoom, feather, threads)
    _check(library, status, "fractal_atlas_composite_rgb")
    return output


def crop_colourise(library, source, source_shape, output_shape, zoom, max_iter, phase, vocal, instrumental, pitch,
                   *, interior=None, accents=None, threads=0) -> np.ndarray:
    """Aurora crop (renderer.h:943-996): ``fractal_crop_colourise``,
    ``_interior`` or ``_accents``."""
    source = np.ascontiguousarray(source, dtype=np.float32)
    width, height = output_shape
    output = np.empty(width * height * 3, dtype=np.uint8)
    common = (source.ctypes.data_as(_c_float_p), source_shape[0], source_shape[1], output.ctypes.data_as(_c_u8_p),
              width, height, zoom, max_iter, phase, vocal, instrumental, pitch)
    if accents is not None:
        accents = np.ascontiguousarray(accents, dtype=np.uint8).reshape(9)
        status = library.fractal_crop_colourise_accents(*common, accents.ctypes.data_as(_c_u8_p),
                                                        *(interior or (0, 0, 0)), threads)
    elif interior is not None:
        status = library.fractal_crop_colourise_interior(*common, *interior, threads)
    else:
        status = library.fractal_crop_colourise(*common, threads)
    _check(library, status, "fractal_crop_colourise")
    return output


def crop_colourise_kfp(library, source, source_shape, output_shape, zoom, max_iter, options, lut,
                       colour=(0.0, 0.0, 0.0, 0.5), threads=0) -> np.ndarray:
    """``fractal_crop_colourise_kfp`` (renderer.h:518-535)."""
    source = np.ascontiguousarray(source, dtype=np.float32)
    lut = np.ascontiguousarray(lut, dtype=np.uint8)
    width, height = output_shape
    output = np.empty(width * height * 3, dtype=np.uint8)
    status = library.fractal_crop_colourise_kfp(
        source.ctypes.data_as(_c_float_p), source_shape[0], source_shape[1], output.ctypes.data_as(_c_u8_p), width,
        height, zoom, max_iter, *colour, ctypes.byref(options), lut.ctypes.data_as(_c_u8_p), lut.shape[0], threads)
    _check(library, status, "fractal_crop_colourise_kfp")
    return output


def colourise_accents(library, field, width, height, max_iter, phase, vocal, instrumental, pitch, accents,
                      interior=(0, 0, 0), threads=0) -> np.ndarray:
    """``fractal_colourise_accents`` (renderer.h:426-440)."""
    field = np.ascontiguousarray(field, dtype=np.float32)
    accents = np.ascontiguousarray(accents, dtype=np.uint8).reshape(9)
    output = np.empty(width * height * 3, dtype=np.uint8)
    status = library.fractal_colourise_accents(
        field.ctypes.data_as(_c_float_p), output.ctypes.data_as(_c_u8_p), width, height, max_iter, phase, vocal,
        instrumental, pitch, accents.ctypes.data_as(_c_u8_p), *interior, threads)
    _check(library, status, "fractal_colourise_accents")
    return output


def stats(library: ctypes.CDLL) -> dict:
    values = (ctypes.c_uint64 * len(EXTENDED_STATS_FIELDS))()
    count = library.fractal_get_last_stats_ex(values, len(EXTENDED_STATS_FIELDS))
    if count < 0:
        raise NativeError(last_error(library))
    return dict(zip(EXTENDED_STATS_FIELDS, (int(v) for v in values[:count])))


def reference_stats(library: ctypes.CDLL, handle: int) -> dict:
    values = (ctypes.c_uint64 * 5)()
    count = library.fractal_get_reference_stats(handle, values, 5)
    if count < 0:
        raise NativeError(last_error(library))
    keys = ("reference_ns", "series_ns", "bla_ns", "series_iteration", "series_order")
    return dict(zip(keys, (int(v) for v in values[:count])))


def iteration_counts(field: np.ndarray, orbit_iteration: np.ndarray, max_iter: int):
    """uint32 iteration counts from a plane render.

    An escaped pixel stores Kalles' raw ``antal`` = n - 1 in ``orbit_iteration``
    (renderer.cpp:8098-8106), so its escape index is orbit_iteration + 1; an
    interior pixel stores max_iter (renderer.cpp:8090).  NaN field values are
    unresolved glitches and are reported as 0.
    """
    counts = np.where(orbit_iteration >= max_iter, max_iter, orbit_iteration + 1)
    counts = counts.astype(np.uint32)
    counts[~np.isfinite(field)] = 0
    return counts
