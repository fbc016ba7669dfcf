"""KFP plane-path parity cases (fractal_colourise_kfp_planes).

The planes are the reference's own render planes of stored parity fields
(orbit_iteration, phase, de_x, de_y, test1, test2), optionally with a seeded
bailout plane, or iteration / transition planes derived from them (a few
transitions negative: hidden glitch pixels).  Options are the named recipes
of the package's KFP module with per-case overrides (phase colour strength,
smoothing method, bailout presets, show_glitches); LUTs are the reference's
(fixtures/kfp_luts.npz).  ``run`` drives any library exporting the ABI.
"""

from __future__ import annotations

import os

import numpy as np

from .runner import _native

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = os.path.join(HERE, "fixtures")
KFP_PLANES_FIXTURE = os.path.join(FIXTURES, "kfp_planes.npz")

FIELDS = {"e100_bias_64x36": (200_000, 400.0), "deep_p80_e32_block32_64x36": (50_000, 0.0),
          "e100_nobla_64x36": (200_000, 0.0), "odd_37x23": (20_000, 0.0)}
SIZES = {"e100_bias_64x36": (64, 36), "deep_p80_e32_block32_64x36": (64, 36), "e100_nobla_64x36": (64, 36),
         "odd_37x23": (37, 23)}


def _case(name, field, recipe, planes="orbit", texture=None, **overrides):
    """`texture` = (width, height, row padding) of a seeded RGB8 texture."""
    return dict(name=name, field=field, recipe=recipe, planes=planes, texture=texture, overrides=overrides)


def texture(spec):
    """(rows of width * 3 + padding bytes, width, height, stride)."""
    width, height, padding = spec
    stride = width * 3 + padding
    rng = np.random.default_rng(width * 1000 + height)
    return rng.integers(0, 256, size=height * stride, dtype=np.uint8), width, height, stride


def kfp_planes_cases() -> list[dict]:
    cases = []
    for field in ("e100_bias_64x36", "deep_p80_e32_block32_64x36", "odd_37x23"):
        for recipe in ("default", "seeded16", "differences7", "method4", "multicolor"):
            cases.append(_case(f"planes_{recipe}_{field}", field, recipe))
    cases += [
        _case("planes_phase_e100_nobla", "e100_nobla_64x36", "seeded16", phase_color_strength=35.0),
        _case("planes_phase_blend_e100_nobla", "e100_nobla_64x36", "multicolor", phase_color_strength=60.0),
        _case("planes_smooth1_e100_nobla", "e100_nobla_64x36", "default", smooth_method=1),
        _case("planes_smooth1_norm3_e100_nobla", "e100_nobla_64x36", "default", smooth_method=1,
              bailout_norm_preset=3, bailout_norm_custom=1.5),
        _case("planes_bailout_plane_e100_nobla", "e100_nobla_64x36", "default", planes="orbit+bailout"),
        _case("planes_iteration_e100_nobla", "e100_nobla_64x36", "seeded16", planes="iteration"),
        _case("planes_iteration_glitches_shown_e100_nobla", "e100_nobla_64x36", "seeded16", planes="iteration",
              show_glitches=1),
        _case("planes_iteration_glitches_hidden_e100_nobla", "e100_nobla_64x36", "seeded16", planes="iteration",
              show_glitches=0),
        _case("planes_de_only_e100_nobla", "e100_nobla_64x36", "differences7", planes="de"),
        _case("planes_texture_e100_bias", "e100_bias_64x36", "default", texture=(50, 40, 7),
              texture_enabled=1, texture_merge=0.6, texture_power=8.0, texture_ratio=50.0),
        _case("planes_texture_strong_deep", "deep_p80_e32_block32_64x36", "seeded16", texture=(64, 36, 0),
              texture_enabled=1, texture_merge=1.0, texture_power=200.0, texture_ratio=100.0),
        _case("planes_texture_iteration_e100_nobla", "e100_nobla_64x36", "differences7", planes="iteration",
              texture=(23, 17, 2), texture_enabled=1, texture_merge=0.35, texture_power=-3.0, texture_ratio=80.0),
        _case("planes_texture_scalar_odd", "odd_37x23", "multicolor", planes="de", texture=(40, 30, 1),
              texture_enabled=1, texture_merge=0.8, texture_power=64.0, texture_ratio=120.0),
        _case("planes_texture_disabled_e100_bias", "e100_bias_64x36", "default", texture=(50, 40, 7),
              texture_enabled=0, texture_merge=0.6, texture_power=8.0, texture_ratio=50.0),
    ]
    return cases


def inputs(case: dict):
    """(field, width, height, max_iter, options, planes dict, lut)."""
    from .make_golden import _package_kfp

    kfp = _package_kfp()
    stored = np.load(os.path.join(FIXTURES, case["field"] + ".npz"))
    max_iter, bias = FIELDS[case["field"]]
    width, height = SIZES[case["field"]]
    options = kfp.options(kfp.recipe(case["recipe"]), field_bias=bias)
    for key, value in case["overrides"].items():
        setattr(options, key, value)
    with np.load(os.path.join(FIXTURES, "kfp_luts.npz")) as luts:
        lut = luts[case["recipe"]]
    orbit = stored["orbit_iteration"].astype(np.int64)
    planes = {}
    if case["planes"].startswith("orbit"):
        planes = {key: stored[key] for key in ("orbit_iteration", "phase", "de_x", "de_y", "test1", "test2")}
        if case["planes"] == "orbit+bailout":
            rng = np.random.default_rng(7)
            bailout = rng.uniform(2.0, 1.0e6, size=orbit.size)
            bailout[rng.uniform(size=orbit.size) < 0.1] = 0.5  # invalid: falls back to the selected radius
            planes["bailout"] = bailout
    elif case["planes"] == "iteration":
        rng = np.random.default_rng(8)
        field = stored["field"].astype(np.float64) + bias
        transition = 1.0 - (field - np.floor(field))
        transition[rng.uniform(size=orbit.size) < 0.05] = -1.0
        planes = {"iteration": np.floor(np.nan_to_num(field, nan=0.0)).astype(np.int64), "transition": transition,
                  "phase": stored["phase"]}
    elif case["planes"] == "de":
        planes = {"de_x": stored["de_x"], "de_y": stored["de_y"]}
    if case["texture"] is not None:
        planes["texture"] = texture(case["texture"])
    return stored["field"], width, height, max_iter, options, planes, lut


def run(library, case: dict) -> np.ndarray:
    native = _native()
    field, width, height, max_iter, options, planes, lut = inputs(case)
    return native.colourise_kfp_planes(library, field, width, height, max_iter, options, planes, lut)
