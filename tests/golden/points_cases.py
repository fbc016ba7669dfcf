"""Point-render parity cases (fractal_render_points[_ex_planes]).

Each case creates a reference at a centre of ``centres.json`` and renders a
seeded list of scaled offsets (mantissa pairs with a shared power-of-two
exponent per point, as the exp-map and glitch-repair layers pass them).
``run`` drives any library exporting the renderer.h ABI: the reference build
(``make_points_golden.py``) and the GB300 library see the same inputs.

The glitch cases put rings of points round the period-80 nucleus at e33,
where every point trips the glitch sentinel: strict renders repair them
exactly (MPFR, both interior and escaping), non-strict ones rebase.
"""

from __future__ import annotations

import math
import os

import numpy as np

from . import cases as case_defs
from .runner import _native

HERE = os.path.dirname(os.path.abspath(__file__))
POINTS_FIXTURE = os.path.join(HERE, "fixtures", "points.npz")


def log_polar(count: int, log10_zoom: float, seed: int, decades: tuple[float, float] = (-1.5, 0.5)):
    """Seeded offsets at radius 10^(-zoom + u), u ~ U(decades), uniform
    angle: (real mantissas, imaginary mantissas, exponents)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(decades[0], decades[1], size=count)
    angle = rng.uniform(0.0, 2.0 * math.pi, size=count)
    log2_radius = (u - log10_zoom) * math.log2(10.0)
    exponents = np.ceil(log2_radius).astype(np.int32)
    magnitude = np.exp2(log2_radius - exponents)
    return magnitude * np.cos(angle), magnitude * np.sin(angle), exponents


def ring(count: int, log10_zoom: float, fraction: float):
    """`count` points on a circle of radius fraction * 10^-zoom."""
    angle = np.linspace(0.0, 2.0 * math.pi, count, endpoint=False)
    mantissa, exponent = math.frexp(fraction * 10.0 ** (-log10_zoom))
    return (mantissa * np.cos(angle), mantissa * np.sin(angle), np.full(count, exponent, dtype=np.int32))


def _case(name, centre, log10_zoom, max_iter, points, *, formula="mandelbrot", julia=None, options=None,
          planes=True):
    return dict(name=name, centre=centre, log10_zoom=log10_zoom, max_iter=max_iter, points=points,
                formula=formula, julia=julia, options=options or {}, planes=planes)


def point_cases() -> list[dict]:
    c = case_defs.centres()
    nucleus = c["deep_nucleus_p80"]
    glitch_points = tuple(np.concatenate(parts) for parts in zip(ring(24, 33.0, 0.5), ring(24, 33.0, 1.0)))
    jf = c["julia_fixed_1"]
    return [
        _case("points_e30_logpolar", c["field_640x360_e30"], 30.0, 50_000, log_polar(512, 30.0, 1)),
        _case("points_e100_logpolar", c["field_e100"], 100.0, 200_000, log_polar(384, 100.0, 2)),
        _case("points_e30_fieldonly", c["field_640x360_e30"], 30.0, 50_000, log_polar(257, 30.0, 3),
              planes=False),
        _case("points_glitch_e33_strict", nucleus, 33.0, 50_000, glitch_points),
        _case("points_glitch_e33_recover", nucleus, 33.0, 50_000, glitch_points,
              options=dict(strict=0, allow_recovery=1)),
        _case("points_julia_e15", dict(re=jf["re"], im=jf["im"]), 15.0, 20_000, log_polar(256, 15.0, 4),
              formula="julia", julia=(jf["c_re"], jf["c_im"])),
        _case("points_burning_ship_e12", c["burning_ship_boundary"], 12.0, 10_000, log_polar(256, 12.0, 5),
              formula="burning-ship"),
        _case("points_tricorn_e12", c["tricorn_boundary"], 12.0, 10_000, log_polar(256, 12.0, 6),
              formula="tricorn"),
    ]


def run(library, case: dict, threads: int = 0) -> dict:
    """Render a case; returns field (f32) and, for planes cases, the six
    planes."""
    native = _native()
    centre = case["centre"]
    x, y = centre["re"], centre["im"]
    zoom = case_defs.zoom_text(case["log10_zoom"]).encode("ascii")
    bits = case_defs.precision_bits(x, y, case["log10_zoom"])
    options = native.RenderOptions(**case["options"])
    julia = case["julia"] or ("0", "0")
    creator_options = options if (case["formula"] != "mandelbrot" or case["options"]) else None
    handle = native.create_reference(library, x, y, zoom, case["max_iter"], bits, 32, formula=case["formula"],
                                     julia=(str(julia[0]), str(julia[1])), options=creator_options)
    try:
        real, imag, exponents = case["points"]
        field, planes = native.render_points(library, handle, zoom, real, imag, exponents, case["max_iter"],
                                             threads=threads, options=options, planes=case["planes"])
    finally:
        library.fractal_destroy_reference(handle)
    result = {"field": field}
    if planes is not None:
        result.update(planes)
    return result
