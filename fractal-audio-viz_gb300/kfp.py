"""Kalles .kfp colour profiles: parsing, the 1024-entry LUT and ABI options.

Host-side mirror of the reference pipeline's profile handling
(visualizer.py): ``KfpPalette`` and ``KALLES_DEFAULT_KFP`` (:302-351,
:430-444), ``_parse_kfp_profile`` (:13341-13441) for the colour-pipeline
fields, ``_kfp_palette_lut`` (:13492-13521), ``NativeKfpOptions.from_profile``
(:1162-1215) and the 3D-relief override ``_kfp_profile_with_3d``
(:13579-13587).  The LUT is built once per profile on the host; the per-pixel
transfer runs in the CUDA library (fractal_colourise_kfp).
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, replace
from typing import Optional

import numpy as np

from . import native


@dataclass(frozen=True)
class KfpProfile:
    stops: tuple
    iter_div: float = 1.0
    color_offset: float = 0.0
    ratio: float = 360.0
    color_method: int = 0
    smooth_method: int = 0
    smooth: bool = True
    flat: bool = False
    inverse_transition: bool = False
    phase_color_strength: float = 0.0
    multi_color: bool = False
    blend_multi_color: bool = False
    multi_colors: tuple = ()
    power: float = 2.0
    slopes: bool = False
    slope_power: float = 50.0
    slope_ratio: float = 50.0
    slope_angle: float = 45.0
    differences: int = 3
    interior_color: tuple = (0, 0, 0)
    show_glitches: bool = True
    bailout_radius_preset: int = 0
    bailout_radius_custom: float = 2.0
    bailout_norm_preset: int = 1
    bailout_norm_custom: float = 2.0


def display_rgb(colour) -> tuple:
    """Kalles serialises colours r,g,b but displays them b,g,r (visualizer.py:13125-13135)."""
    return (int(colour[2]), int(colour[1]), int(colour[0]))


def _fields(text: str) -> dict:
    fields = {}
    for line in text.splitlines():
        if ":" not in line:
            continue
        key, value = line.split(":", 1)
        fields[key.strip().casefold()] = value.strip()
    return fields


def _number(fields, key, default, cast=float):
    value = fields.get(key.casefold())
    if value is None or not value.strip():
        return cast(default)
    token = value.replace(",", " ").split()[0]
    return cast(float(token)) if cast is int else cast(token)


def parse_kfp(text: str) -> KfpProfile:
    """Colour-pipeline fields of a .kfp file (camera and formula fields are
    ignored, as Kalles does when loading a palette)."""
    fields = _fields(text)
    values = [int(v) for v in fields["colors"].replace(";", ",").split(",") if v.strip()]
    if len(values) >= 7 and 2 <= values[0] and len(values) == 1 + values[0] * 3:
        values = values[1:]
    if len(values) < 6 or len(values) % 3:
        raise ValueError("KFP Colors field needs at least two complete RGB stops")
    stops = tuple(display_rgb(values[i:i + 3]) for i in range(0, len(values), 3))
    interior = [int(v) for v in fields.get("interiorcolor", "0,0,0").rstrip(" ,;").split(",")]
    offset = int(_number(fields, "ColorOffset", 0, float))
    multi = []
    for entry in fields.get("multicolors", "").replace(";", " ").split():
        parts = [p for p in entry.split(",") if p]
        if len(parts) == 3:
            multi.append((float(parts[0]), int(parts[1]), int(parts[2])))
    return KfpProfile(
        stops=stops,
        iter_div=_number(fields, "IterDiv", 1.0),
        color_offset=float(offset if 0 <= offset <= 1023 else 0),
        ratio=_number(fields, "Ratio", 360.0),
        color_method=int(_number(fields, "ColorMethod", 0)),
        smooth=bool(int(_number(fields, "Smooth", 1))),
        flat=bool(int(_number(fields, "Flat", 0))),
        inverse_transition=bool(int(_number(fields, "InverseTransition", 0))),
        phase_color_strength=_number(fields, "ColorPhaseStrength", 0.0),
        multi_color=bool(int(_number(fields, "MultiColor", 0))),
        blend_multi_color=bool(int(_number(fields, "BlendMC", 0))),
        multi_colors=tuple(multi),
        slopes=bool(int(_number(fields, "Slopes", 0))),
        slope_power=float(int(_number(fields, "SlopePower", 50))),
        slope_ratio=float(int(_number(fields, "SlopeRatio", 50))),
        slope_angle=float(int(_number(fields, "SlopeAngle", 45))),
        differences=int(_number(fields, "Differences", 0)),
        interior_color=display_rgb(interior),
        show_glitches=bool(int(_number(fields, "ShowGlitches", 1))),
    )


# Kalles' own default palette settings with its key colours (the bundled
# palettes/kalles-default.kfp recipe).
KALLES_DEFAULT_COLORS = (255, 255, 255, 128, 0, 64, 160, 0, 0, 192, 128, 0, 64, 128, 0, 0, 255, 255,
                         64, 128, 255, 0, 0, 255)
KALLES_DEFAULT = KfpProfile(
    stops=tuple(display_rgb(KALLES_DEFAULT_COLORS[i:i + 3]) for i in range(0, len(KALLES_DEFAULT_COLORS), 3)),
    iter_div=0.01,
    ratio=360.0,
    color_method=7,
    smooth_method=0,
    smooth=True,
    power=2.0,
    slopes=True,
    slope_power=50.0,
    slope_ratio=20.0,
    slope_angle=45.0,
    differences=3,
    interior_color=(0, 0, 0),
)


def with_relief(profile: KfpProfile, enabled: Optional[bool]) -> KfpProfile:
    """The 3D-relief switch is the slopes override (visualizer.py:13579-13587)."""
    return profile if enabled is None else replace(profile, slopes=bool(enabled))


def palette_lut(profile: KfpProfile, size: int = 1024) -> np.ndarray:
    """Cyclic sine interpolation of the key colours into ``size`` RGB8 entries.

    Position i spans the stops cyclically; the blend fraction is the
    half-period sine ease sin((f - 1/2) pi)/2 + 1/2, formed in float64, and
    each channel is truncated to a byte.
    """
    size = max(2, int(size))
    stops = np.asarray(profile.stops, dtype=np.float64)
    if stops.shape[0] < 2:
        raise ValueError("KFP palette needs at least two colour stops")
    position = np.arange(size, dtype=np.float64) * float(stops.shape[0]) / float(size)
    left = np.floor(position).astype(np.intp)
    right = (left + 1) % stops.shape[0]
    fraction = position - left.astype(np.float64)
    fraction = np.sin((fraction - 0.5) * np.pi) / 2.0 + 0.5
    lut = stops[left] * (1.0 - fraction[:, None]) + stops[right] * fraction[:, None]
    return np.ascontiguousarray(np.clip(lut, 0.0, 255.0).astype(np.uint8))


def options(profile: KfpProfile, field_bias: float = 0.0) -> native.KfpOptions:
    """``FractalKfpOptions`` for a profile (NativeKfpOptions.from_profile)."""
    if len(profile.multi_colors) > native.KFP_MAX_MULTI_COLORS:
        raise ValueError("KFP profile contains too many multi-colour waves")
    field_bias = float(field_bias)
    if not math.isfinite(field_bias) or field_bias < 0.0:
        raise ValueError("KFP field bias must be finite and non-negative")
    o = native.KfpOptions()
    o.struct_size = ctypes.sizeof(native.KfpOptions)
    o.version = native.KFP_OPTIONS_VERSION
    o.iter_div = profile.iter_div
    o.color_offset = profile.color_offset
    o.ratio = profile.ratio
    o.color_method = profile.color_method
    o.smooth_method = profile.smooth_method
    o.smooth = int(profile.smooth)
    o.flat = int(profile.flat)
    o.inverse_transition = int(profile.inverse_transition)
    o.phase_color_strength = profile.phase_color_strength
    o.multi_color = int(profile.multi_color)
    o.blend_multi_color = int(profile.blend_multi_color)
    o.multi_color_count = len(profile.multi_colors)
    for i, (period, start, kind) in enumerate(profile.multi_colors):
        o.multi_color_period[i] = period
        o.multi_color_start[i] = start
        o.multi_color_type[i] = kind
    o.power = profile.power
    o.slopes = int(profile.slopes)
    o.slope_power = profile.slope_power
    o.slope_ratio = profile.slope_ratio
    o.slope_angle = profile.slope_angle
    o.differences = profile.differences
    o.interior_color[:] = profile.interior_color
    o.field_bias = field_bias
    o.bailout_radius_preset = profile.bailout_radius_preset
    o.bailout_radius_custom = profile.bailout_radius_custom
    o.bailout_norm_preset = profile.bailout_norm_preset
    o.bailout_norm_custom = profile.bailout_norm_custom
    o.texture_enabled = 0
    o.texture_merge = 1.0
    o.texture_power = 200.0
    o.texture_ratio = 100.0
    o.texture_resize = 1
    o.use_opengl = 0
    o.use_srgb = 0
    o.show_glitches = int(profile.show_glitches)
    return o


def seeded_profile(seed: int, stops: int = 16) -> KfpProfile:
    """A .kfp-style recipe with ``stops`` seeded key colours: distance
    transfer (ColorMethod 7, Differences 3), slopes (3D relief) on, dither
    (always applied by the transfer)."""
    rng = np.random.default_rng(seed)
    colours = tuple(tuple(int(v) for v in rng.integers(0, 256, size=3)) for _ in range(stops))
    return replace(KALLES_DEFAULT, stops=colours)


def colourise(library, field: np.ndarray, width: int, height: int, max_iter: int, profile: KfpProfile,
              *, field_bias: float = 0.0, lut: Optional[np.ndarray] = None, threads: int = 0) -> np.ndarray:
    """fractal_colourise_kfp through the ABI into host RGB8."""
    field = np.ascontiguousarray(field, dtype=np.float32)
    lut = palette_lut(profile) if lut is None else np.ascontiguousarray(lut, dtype=np.uint8)
    out = np.empty(width * height * 3, dtype=np.uint8)
    opts = options(profile, field_bias)
    status = library.fractal_colourise_kfp(
        field.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
        width, height, max_iter, 0.0, 0.0, 0.0, 0.5, ctypes.byref(opts),
        lut.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), lut.shape[0], threads)
    if status != 0:
        raise native.NativeError(native.last_error(library))
    return out


def recipe(name: str) -> KfpProfile:
    """Named test and benchmark recipes (variations of the Kalles default)."""
    if name == "default":
        return KALLES_DEFAULT
    if name == "seeded16":
        return seeded_profile(4242, 16)
    if name == "multicolor":
        return replace(seeded_profile(77, 6), multi_color=True, blend_multi_color=True,
                       multi_colors=((120.0, 0, 0), (-80.0, 0, 1), (300.0, 0, 2), (45.0, 0, 2)))
    if name == "flat_nosmooth":
        return replace(KALLES_DEFAULT, flat=True, smooth=False, color_method=0, iter_div=1.0)
    if name == "inverse":
        return replace(seeded_profile(5, 9), inverse_transition=True, color_method=0, iter_div=0.37,
                       color_offset=100.0)
    if name.startswith("method"):
        return replace(KALLES_DEFAULT, color_method=int(name[6:]), iter_div=0.05)
    if name.startswith("differences"):
        return replace(KALLES_DEFAULT, differences=int(name[11:]))
    raise KeyError(name)
