"""Atlas compositor parity cases (fractal_atlas_field[_ex], fractal_atlas_colourise[_interior|_accents],
fractal_atlas_colourise_kfp_raw, fractal_crop_field, fractal_crop_rgb, fractal_atlas_composite_rgb,
fractal_crop_colourise[_interior|_accents], fractal_crop_colourise_kfp, fractal_colourise_accents).

Each case names its parent and child fields (stored golden fields of
``fixtures/`` or seeded synthetic fields with interior, NaN and +inf
samples), the output size and the call's arguments.  ``run`` drives any
library exporting the renderer.h atlas ABI, so the reference build (fixture
generation, ``make_atlas_golden.py``) and the GB300 library see the same
inputs.
"""

from __future__ import annotations

import os

import numpy as np

from . import cases as case_defs
from .runner import _native

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = os.path.join(HERE, "fixtures")
ATLAS_FIXTURE = os.path.join(FIXTURES, "atlas.npz")

COLOUR = (0.3, 0.4, 0.7, 0.5)  # phase, vocal, instrumental, pitch
ACCENTS = (250, 40, 10, 20, 230, 90, 30, 60, 250)


def synthetic_field(width: int, height: int, max_iter: int, seed: int, bias: float = 0.0) -> np.ndarray:
    """Seeded smooth values in [0, cap) with 15 % interior (cap - bias),
    4 % NaN (unresolved glitch) and 1 % +inf samples."""
    rng = np.random.default_rng(seed)
    values = rng.uniform(0.0, max_iter - bias, size=width * height).astype(np.float32)
    kind = rng.uniform(size=width * height)
    values[kind < 0.15] = np.float32(max_iter - bias)
    values[(kind >= 0.15) & (kind < 0.19)] = np.nan
    values[(kind >= 0.19) & (kind < 0.20)] = np.inf
    return values


def synthetic_rgb(width: int, height: int, seed: int) -> np.ndarray:
    """Seeded RGB8 image: smooth gradients plus noise (a coloured keyframe
    stand-in for the RGB compositor)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    channels = [127.5 + 127.5 * np.sin(x / (7.0 + 13 * rng.uniform()) + y / (11.0 + 5 * rng.uniform()) + k)
                for k in range(3)]
    image = np.stack(channels, axis=-1) + rng.normal(0.0, 12.0, size=(height, width, 3))
    return np.clip(np.rint(image), 0, 255).astype(np.uint8).reshape(-1)


def _stored(name: str):
    case = next(c for c in case_defs.parity_cases() + case_defs.alternate_cases() if c["name"] == name)
    field = np.load(os.path.join(FIXTURES, name + ".npz"))["field"].astype(np.float32)
    return field, (case["width"], case["height"]), case["max_iter"]


def source(spec):
    """(field, (width, height), max_iter) for a stored name or a synthetic
    tuple ("synthetic", width, height, max_iter, seed[, bias])."""
    if spec is None:
        return None, None, 0
    if isinstance(spec, str):
        return _stored(spec)
    if spec[0] == "rgb":
        _, width, height, seed = spec
        return synthetic_rgb(width, height, seed), (width, height), 0
    _, width, height, max_iter, seed, *rest = spec
    bias = rest[0] if rest else 0.0
    return synthetic_field(width, height, max_iter, seed, bias), (width, height), max_iter


def _case(name, kind, parent, child, output, parent_zoom, fraction, palette, **extra):
    return dict(name=name, kind=kind, parent=parent, child=child, output=output, parent_zoom=parent_zoom,
                fraction=fraction, palette=palette, **extra)


CASES = [
    # Scalar frames.
    _case("field_levels_13_14", "field", "fhd_level13_128x72", "fhd_level14_128x72", (160, 90), 1.6, 0.55, 1000),
    _case("field_ex_bias", "field", ("synthetic", 97, 53, 3000, 11, 2.5), ("synthetic", 64, 40, 5000, 12, 4.0),
          (211, 117), 2.3, 0.47, 2000, child_zoom=1.4, parent_bias=2.5, child_bias=4.0, output_bias=1.5,
          feather=12),
    _case("field_ex_interior", "field", "fhd_level00_128x72", "fhd_level05_128x72", (192, 108), 1.3, 0.62, 100,
          child_zoom=1.0, parent_bias=0.0, child_bias=0.0, output_bias=0.0, feather=48),
    _case("field_ex_full_child", "field", "fhd_level00_128x72", "fhd_level05_128x72", (128, 72), 1.0, 1.0, 100,
          child_zoom=1.7, parent_bias=0.0, child_bias=0.0, output_bias=3.0, feather=48),
    _case("field_ex_no_child", "field", "fhd_level05_128x72", None, (256, 144), 1.0, 0.0, 100,
          child_zoom=1.0, parent_bias=0.0, child_bias=0.0, output_bias=0.0, feather=48),
    _case("field_ex_narrow_child", "field", "fhd_level13_128x72", "fhd_level14_128x72", (150, 100), 8.0, 0.02,
          100, child_zoom=1.0, parent_bias=0.0, child_bias=0.0, output_bias=0.0, feather=48),
    _case("field_ex_no_feather", "field", "fhd_level13_128x72", "fhd_level14_128x72", (150, 100), 1.1, 0.5,
          100, child_zoom=1.0, parent_bias=0.0, child_bias=0.0, output_bias=0.0, feather=0),
    _case("field_glitch_parent", "field", "deep_p80_e34_glitch_64x36", "deep_p80_e34_recover_64x36", (100, 60),
          1.2, 0.7, 100),
    _case("field_synthetic_mix", "field", ("synthetic", 97, 53, 3000, 21), ("synthetic", 50, 31, 3000, 22),
          (173, 91), 1.9, 0.71, 3000),
    # Aurora frames.
    _case("colour_levels_13_14", "colour", "fhd_level13_128x72", "fhd_level14_128x72", (160, 90), 1.6, 0.55, 1000),
    _case("colour_interior_pitch", "colour", "fhd_level00_128x72", "fhd_level05_128x72", (333, 187), 1.45, 0.8,
          0, pitch=0.9, interior=(12, 200, 77)),
    _case("colour_accents", "colour", "fhd_level00_128x72", "fhd_level05_128x72", (240, 135), 2.0, 0.5, 20000,
          interior=(5, 5, 5), accents=ACCENTS, pitch=0.2),
    _case("colour_full_child", "colour", "fhd_level13_128x72", "fhd_level14_128x72", (128, 72), 1.0, 1.0, 0),
    _case("colour_no_child", "colour", "fhd_level22_128x72", None, (300, 170), 3.0, 0.0, 0),
    _case("colour_glitch_parent", "colour", "deep_p80_e34_glitch_64x36", "deep_p80_e34_recover_64x36", (100, 60),
          1.2, 0.7, 0),
    _case("colour_synthetic_mix", "colour", ("synthetic", 97, 53, 3000, 31), ("synthetic", 50, 31, 3000, 32),
          (173, 91), 1.9, 0.71, 100, interior=(40, 41, 42)),
    # Raw KFP frames (one scalar surface, one KFP pass).
    _case("kfp_raw_levels_13_14", "kfp_raw", "fhd_level13_128x72", "fhd_level14_128x72", (320, 180), 1.7, 0.55,
          0, child_zoom=1.0, recipe="seeded16", max_iter=42639, field_bias=0.0),
    _case("kfp_raw_interior_zoomed_child", "kfp_raw", "fhd_level00_128x72", "fhd_level05_128x72", (256, 144), 1.3,
          0.62, 0, child_zoom=1.6, recipe="default", max_iter=18255, field_bias=0.0),
    _case("kfp_raw_centred", "kfp_raw", "fhd_level00_128x72", "fhd_level05_128x72", (250, 141), 2.2, 0.4, 0,
          child_zoom=1.0, recipe="seeded16", max_iter=18255, field_bias=18255.0, centred=True),
    _case("kfp_raw_full_child", "kfp_raw", "fhd_level13_128x72", "fhd_level14_128x72", (200, 112), 1.0, 1.0, 0,
          child_zoom=1.25, recipe="method4", max_iter=42639, field_bias=0.0),
    _case("kfp_raw_no_child", "kfp_raw", "fhd_level22_128x72", None, (192, 108), 2.5, 0.0, 0, child_zoom=1.0,
          recipe="differences7", max_iter=64313, field_bias=0.0),
    _case("kfp_raw_synthetic_bias", "kfp_raw", ("synthetic", 97, 53, 3000, 41), ("synthetic", 50, 31, 3000, 42),
          (173, 91), 1.9, 0.71, 0, child_zoom=1.1, recipe="multicolor", max_iter=3000, field_bias=0.5,
          centred=True),
    _case("kfp_raw_inexact_bias", "kfp_raw", "fhd_level13_128x72", "fhd_level14_128x72", (180, 101), 1.45, 0.66,
          0, child_zoom=1.0, recipe="seeded16", max_iter=42639, field_bias=1234.1, centred=True),
    # Crops of one field or image, and the RGB compositor.
    _case("crop_field_zoom", "crop_field", "fhd_level22_128x72", None, (301, 173), 1.8, 0.0, 0),
    _case("crop_field_glitch", "crop_field", "deep_p80_e34_recover_64x36", None, (97, 55), 1.0, 0.0, 0),
    _case("crop_rgb_zoom", "crop_rgb", ("rgb", 160, 90, 51), None, (333, 187), 2.3, 0.0, 0),
    _case("crop_rgb_identity", "crop_rgb", ("rgb", 160, 90, 52), None, (160, 90), 0.5, 0.0, 0),
    _case("composite_rgb", "composite_rgb", ("rgb", 160, 90, 53), ("rgb", 128, 72, 54), (320, 180), 1.9, 0.52, 0,
          child_zoom=1.2, feather=24),
    _case("composite_rgb_full", "composite_rgb", ("rgb", 160, 90, 55), ("rgb", 128, 72, 56), (200, 113), 1.0, 1.0,
          0, child_zoom=1.0, feather=100),
    _case("composite_rgb_no_child", "composite_rgb", ("rgb", 160, 90, 57), None, (200, 113), 1.4, 0.0, 0,
          child_zoom=1.0, feather=0),
    _case("crop_colour", "crop_colour", "fhd_level00_128x72", None, (250, 141), 1.6, 0.0, 0, max_iter=4709),
    _case("crop_colour_interior_accents", "crop_colour", "fhd_level05_128x72", None, (180, 101), 2.4, 0.0, 0,
          max_iter=18255, interior=(30, 20, 10), accents=ACCENTS, pitch=0.8),
    _case("crop_colour_interior", "crop_colour", ("synthetic", 97, 53, 3000, 61), None, (173, 91), 1.2, 0.0, 0,
          max_iter=3000, interior=(1, 2, 3)),
    _case("crop_kfp", "crop_kfp", "fhd_level13_128x72", None, (240, 135), 1.5, 0.0, 0, recipe="seeded16",
          max_iter=39929, field_bias=0.0),
    _case("crop_kfp_bias", "crop_kfp", "e100_bias_64x36", None, (128, 72), 1.25, 0.0, 0, recipe="default",
          max_iter=200000, field_bias=400.0),
    # Single-field accent colour.
    _case("colourise_accents_level22", "accents", "fhd_level22_128x72", None, (128, 72), 1.0, 0.0, 0,
          interior=(9, 8, 7), accents=ACCENTS, pitch=0.75),
]


def kfp_inputs(case: dict):
    """(KfpOptions, LUT) of a raw KFP case: the options block from the
    package's profile recipes, the LUT the reference's Python built for that
    recipe (fixtures/kfp_luts.npz)."""
    from .make_golden import _package_kfp

    kfp = _package_kfp()
    with np.load(os.path.join(FIXTURES, "kfp_luts.npz")) as luts:
        lut = luts[case["recipe"]]
    return kfp.options(kfp.recipe(case["recipe"]), field_bias=case["field_bias"]), lut


def inputs(case: dict):
    """(parent, parent_shape, parent_cap, child, child_shape, child_cap) of a
    case: its sources, or explicit ``arrays`` = ((field, shape, cap), (field,
    shape, cap) or None); ``centred`` stores each source relative to its own
    cap (the centred encoding)."""
    if "arrays" in case:
        (parent, parent_shape, parent_cap), child_spec = case["arrays"]
        child, child_shape, child_cap = child_spec if child_spec is not None else (None, None, 0)
    else:
        parent, parent_shape, parent_cap = source(case["parent"])
        child, child_shape, child_cap = source(case["child"])
    if case.get("centred"):
        parent = (parent - np.float32(parent_cap)).astype(np.float32)
        if child is not None:
            child = (child - np.float32(child_cap)).astype(np.float32)
    return parent, parent_shape, parent_cap, child, child_shape, child_cap


def run(library, case: dict) -> np.ndarray:
    native = _native()
    parent, parent_shape, parent_cap, child, child_shape, child_cap = inputs(case)
    if case["kind"] == "crop_field":
        return native.crop_field(library, parent, parent_shape, case["output"], case["parent_zoom"])
    if case["kind"] == "crop_rgb":
        return native.crop_rgb(library, parent, parent_shape, case["output"], case["parent_zoom"])
    if case["kind"] == "composite_rgb":
        return native.atlas_composite_rgb(library, parent, parent_shape, child, child_shape, case["output"],
                                          case["parent_zoom"], case["fraction"], case["child_zoom"],
                                          case["feather"])
    if case["kind"] == "crop_colour":
        phase, vocal, instrumental, pitch = COLOUR
        return native.crop_colourise(library, parent, parent_shape, case["output"], case["parent_zoom"],
                                     case["max_iter"], phase, vocal, instrumental, case.get("pitch", pitch),
                                     interior=case.get("interior"), accents=case.get("accents"))
    if case["kind"] == "crop_kfp":
        options, lut = kfp_inputs(case)
        return native.crop_colourise_kfp(library, parent, parent_shape, case["output"], case["parent_zoom"],
                                         case["max_iter"], options, lut)
    if case["kind"] == "kfp_raw":
        options, lut = kfp_inputs(case)
        return native.atlas_colourise_kfp_raw(library, parent, parent_shape, parent_cap, child, child_shape,
                                              child_cap, case["output"], case["parent_zoom"], case["fraction"],
                                              case["child_zoom"], case["max_iter"], options, lut)
    phase, vocal, instrumental, pitch = COLOUR
    pitch = case.get("pitch", pitch)
    if case["kind"] == "accents":
        width, height = parent_shape
        return native.colourise_accents(library, parent, width, height, parent_cap, phase, vocal, instrumental,
                                        pitch, case["accents"], case.get("interior", (0, 0, 0)))
    if case["kind"] == "field":
        return native.atlas_field(library, parent, parent_shape, parent_cap, child, child_shape, child_cap,
                                  case["output"], case["parent_zoom"], case["fraction"], case["palette"],
                                  child_zoom=case.get("child_zoom"), parent_bias=case.get("parent_bias"),
                                  child_bias=case.get("child_bias"), output_bias=case.get("output_bias"),
                                  feather=case.get("feather"))
    return native.atlas_colourise(library, parent, parent_shape, parent_cap, child, child_shape, child_cap,
                                  case["output"], case["parent_zoom"], case["fraction"], case["palette"], phase,
                                  vocal, instrumental, pitch, interior=case.get("interior"),
                                  accents=case.get("accents"))
