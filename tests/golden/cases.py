"""Parity cases shared by the fixture generator, the tests and the bench.

Each case is a plain dict describing one call sequence through the
renderer.h ABI.  ``kind``:
  * ``reference``  reusable reference (creator + optional tier clone), then
                   fractal_render_reference_ex_planes  (atlas path,
                   visualizer.py:6250-6600)
  * ``oneshot``    render_fractal_ex_planes with use_perturbation=1
                   (visualizer.py:6126-6248, series order 8 / block 32)
  * ``direct``     render_fractal_ex_planes with use_perturbation=0

Centres come from centres.json (seeded Misiurewicz points and Julia
boundary constants, see make_centres.py).
"""

from __future__ import annotations

import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def centres() -> dict:
    with open(os.path.join(HERE, "centres.json"), encoding="ascii") as handle:
        return json.load(handle)


def precision_bits(x: str, y: str, log10_zoom: float) -> int:
    """MPFR precision the reference pipeline asks for (visualizer.py:5003-5036)."""

    def fractional_places(text: str) -> int:
        text = text.strip().lstrip("+-")
        return len(text.split(".", 1)[1]) if "." in text else 0

    digits = max(50, 32 + int(math.ceil(max(0.0, log10_zoom))), fractional_places(x), fractional_places(y))
    return max(256, int(digits * math.log2(10.0)) + 32)


def zoom_text(log10_zoom: float) -> str:
    exponent = math.floor(log10_zoom)
    mantissa = 10.0 ** (log10_zoom - exponent)
    return f"{mantissa:.17g}e{exponent:+d}"


def atlas_cap(level: int, factor: float = 8.0) -> int:
    """Iteration cap of atlas level i: 2000 + 3000 per decade, capped at 200k
    (visualizer.py:6958-6979 with the per-tile zoom (i+1)*log10(factor))."""
    log_zoom = min(50.0, (level + 1) * math.log10(factor))
    return min(200_000, max(64, int(2000 + 3000 * max(0.0, log_zoom))))


def fhd_stack_levels(count: int = 55, factor: float = 8.0):
    """Atlas keyframe levels: (level, log10 zoom, cap) for the FHD stack."""
    step = math.log10(factor)
    return [(i, i * step, atlas_cap(i, factor)) for i in range(count)]


def _m(name, **kw):
    base = dict(name=name, formula="mandelbrot", options={}, series_order=3, series_block=256,
                image_series_order=32, compare="exact")
    base.update(kw)
    return base


def parity_cases() -> list[dict]:
    c = centres()
    e30 = c["field_640x360_e30"]
    e50 = c["fhd_stack_e50"]
    e100 = c["field_e100"]
    julia = c["julia_c"]
    cases = [
        # The 640x360 e30 field, cap 50k (full size; stored as hashes).
        _m("e30_640x360", kind="reference", centre=e30, log10_zoom=30.0, width=640, height=360,
           max_iter=50_000, store="hash"),
        _m("e30_160x90", kind="reference", centre=e30, log10_zoom=30.0, width=160, height=90,
           max_iter=50_000),
        _m("e30_oneshot_96x54", kind="oneshot", centre=e30, log10_zoom=30.0, width=96, height=54,
           max_iter=50_000),
        _m("e100_128x72", kind="reference", centre=e100, log10_zoom=100.0, width=128, height=72,
           max_iter=200_000),
        _m("e100_kalles_96x54", kind="reference", centre=e100, log10_zoom=100.0, width=96, height=54,
           max_iter=200_000, options=dict(escape_radius_mode=1, coordinate_mode=1)),
        _m("e100_nobla_64x36", kind="reference", centre=e100, log10_zoom=100.0, width=64, height=36,
           max_iter=200_000, options=dict(disable_bla=1)),
        _m("e100_nonstrict_64x36", kind="reference", centre=e100, log10_zoom=100.0, width=64, height=36,
           max_iter=200_000, options=dict(strict=0, allow_recovery=1)),
        _m("e100_order1_64x36", kind="reference", centre=e100, log10_zoom=100.0, width=64, height=36,
           max_iter=200_000, series_order=1),
        _m("e100_bias_64x36", kind="reference", centre=e100, log10_zoom=100.0, width=64, height=36,
           max_iter=200_000, options=dict(output_bias=400.0)),
        # Views beside deep minibrots on the e100 point's spiral: BLA blocks
        # (cubic and linear), double tails, rebases and glitch sentinels.
        _m("deep_p80_e32_96x54", kind="reference", centre=c["deep_nucleus_p80"], log10_zoom=32.3, width=96,
           height=54, max_iter=50_000, root_log10_zoom=31.0, clone=True),
        _m("deep_p70_e28_linear_96x54", kind="reference", centre=c["deep_nucleus_p70"], log10_zoom=28.3,
           width=96, height=54, max_iter=50_000, root_log10_zoom=27.0, clone=True, series_order=1),
        _m("deep_p70_e28_quadratic_64x36", kind="reference", centre=c["deep_nucleus_p70"], log10_zoom=28.3,
           width=64, height=36, max_iter=50_000, root_log10_zoom=27.0, clone=True, series_order=2),
        _m("deep_p80_e34_glitch_64x36", kind="reference", centre=c["deep_nucleus_p80"], log10_zoom=34.5,
           width=64, height=36, max_iter=50_000, root_log10_zoom=33.0, clone=True),
        _m("deep_p80_e34_recover_64x36", kind="reference", centre=c["deep_nucleus_p80"], log10_zoom=34.5,
           width=64, height=36, max_iter=50_000, root_log10_zoom=33.0, clone=True,
           options=dict(strict=0, allow_recovery=1)),
        _m("deep_p80_e32_block32_64x36", kind="reference", centre=c["deep_nucleus_p80"], log10_zoom=32.3,
           width=64, height=36, max_iter=50_000, root_log10_zoom=31.0, clone=True, series_block=32),
        _m("odd_1x1", kind="reference", centre=e100, log10_zoom=60.0, width=1, height=1, max_iter=20_000),
        _m("odd_3x5", kind="reference", centre=e100, log10_zoom=60.0, width=3, height=5, max_iter=20_000),
        _m("odd_37x23", kind="reference", centre=e30, log10_zoom=20.0, width=37, height=23,
           max_iter=20_000),
    ]
    cases += deep_mandelbrot_cases()
    # FHD keyframe stack: a reduced-size sample of its levels.  Levels below
    # 1e12 take the direct path exactly as the atlas does
    # (visualizer.py:6152); deeper levels use the reference path with the
    # root reference prepared at the stack's maximum depth and a tier clone
    # at the level's own zoom.
    levels = fhd_stack_levels()
    deepest = levels[-1][1]
    for level, log_zoom, cap in [levels[i] for i in (0, 5, 13, 14, 22, 33, 44, 54)]:
        if log_zoom < 12.0:
            cases.append(_m(f"fhd_level{level:02d}_128x72", kind="direct", centre=e50, log10_zoom=log_zoom,
                            width=128, height=72, max_iter=cap))
        else:
            cases.append(_m(f"fhd_level{level:02d}_128x72", kind="reference", centre=e50, log10_zoom=log_zoom,
                            width=128, height=72, max_iter=cap, root_log10_zoom=deepest,
                            root_max_iter=levels[-1][2], clone=True))
    # Direct path for the other formulas.
    for formula in ("julia", "burning-ship", "tricorn"):
        cases.append(_m(f"direct_{formula}_96x54", kind="direct", formula=formula,
                        centre=dict(re="0.0", im="0.0") if formula == "julia" else e30,
                        julia=(float(julia[0]["re"]), float(julia[0]["im"])), log10_zoom=0.2,
                        width=96, height=54, max_iter=4000))
    return cases


def alternate_cases() -> list[dict]:
    """Deep fields of the other formulas (render_alternate_reference_impl).

    Julia views centre on the repelling fixed point of z^2 + c (the
    reference pipeline's Julia zoom target, recovered in MPFR); burning-ship
    and tricorn views centre on seeded parameter-set boundary points.
    """
    c = centres()
    cases = []
    for key in ("julia_fixed_1", "julia_fixed_2"):
        jf = c[key]
        for log_zoom, size in ((9.0, (96, 54)), (15.0, (64, 36))):
            cases.append(_m(f"{key}_e{int(log_zoom)}_{size[0]}x{size[1]}", kind="reference", formula="julia",
                            centre=dict(re=jf["re"], im=jf["im"]), julia=(jf["c_re"], jf["c_im"]),
                            log10_zoom=log_zoom, width=size[0], height=size[1], max_iter=20_000))
    for formula, key in (("burning-ship", "burning_ship_boundary"), ("tricorn", "tricorn_boundary")):
        for log_zoom, size in ((7.0, (96, 54)), (12.0, (64, 36))):
            cases.append(_m(f"{formula}_e{int(log_zoom)}_{size[0]}x{size[1]}", kind="reference", formula=formula,
                            centre=c[key], log10_zoom=log_zoom, width=size[0], height=size[1], max_iter=10_000))
    cases.extend(deep_alternate_cases())
    # Non-strict (cycle detection) and linear-block-free variants.
    jf = c["julia_fixed_1"]
    cases.append(_m("julia_fixed_1_nonstrict_64x36", kind="reference", formula="julia",
                    centre=dict(re=jf["re"], im=jf["im"]), julia=(jf["c_re"], jf["c_im"]), log10_zoom=9.0,
                    width=64, height=36, max_iter=20_000, options=dict(strict=0)))
    cases.append(_m("burning-ship_nobla_48x27", kind="reference", formula="burning-ship",
                    centre=c["burning_ship_boundary"], log10_zoom=7.0, width=48, height=27, max_iter=10_000,
                    options=dict(disable_bla=1)))
    return cases


# Depths and caps of the deep alternate-formula fixtures: the batch
# workload's range (zoom 1e10-1e100, caps 1e4-1e6) on small fields.
DEEP_ALTERNATE_LEVELS = ((30.0, 100_000), (60.0, 300_000), (100.0, 1_000_000))


def deep_mandelbrot_cases() -> list[dict]:
    """Mandelbrot views deeper than 1e100: 1e300 (deltas near the bottom of
    the double exponent range) on the 360-digit e100 centre and 1e1000
    (beyond it: only the extended-exponent arithmetic represents them) on a
    1060-digit centre; cap 50,000, 64x36."""
    c = centres()
    return [
        _m("e300_64x36", kind="reference", centre=c["field_e100"], log10_zoom=300.0, width=64, height=36,
           max_iter=50_000),
        _m("e1000_64x36", kind="reference", centre=c["field_e1000"], log10_zoom=1000.0, width=64, height=36,
           max_iter=50_000),
    ]


def deep_alternate_cases() -> list[dict]:
    """Julia, burning-ship and tricorn fields at 1e30, 1e60 and 1e100 with
    caps 1e5-1e6 (64x36): Julia on the repelling fixed point, the others on
    130-digit seeded preperiodic parameters."""
    c = centres()
    cases = []
    jf = c["julia_fixed_1"]
    for log_zoom, cap in DEEP_ALTERNATE_LEVELS:
        cases.append(_m(f"julia_fixed_1_deep_e{int(log_zoom)}_64x36", kind="reference", formula="julia",
                        centre=dict(re=jf["re"], im=jf["im"]), julia=(jf["c_re"], jf["c_im"]), log10_zoom=log_zoom,
                        width=64, height=36, max_iter=cap))
    for formula, key in (("burning-ship", "burning_ship_deep"), ("tricorn", "tricorn_deep")):
        for log_zoom, cap in DEEP_ALTERNATE_LEVELS:
            cases.append(_m(f"{formula}_deep_e{int(log_zoom)}_64x36", kind="reference", formula=formula,
                            centre=c[key], log10_zoom=log_zoom, width=64, height=36, max_iter=cap))
    return cases


def kfp_cases() -> list[dict]:
    """KFP colour cases: (field fixture, profile recipe, max_iter, field_bias).

    Profiles are named recipes built by fractal-audio-viz_gb300/kfp.py; the
    fields are stored parity fixtures, so the colour pass is tested on the
    reference's own scalar fields.
    """
    cases = []
    fields = [("e30_160x90", 50_000, 0.0), ("fhd_level00_128x72", 4709, 0.0), ("deep_p80_e32_96x54", 50_000, 0.0),
              ("e100_bias_64x36", 200_000, 400.0), ("odd_37x23", 20_000, 0.0), ("odd_3x5", 20_000, 0.0)]
    recipes = ["default", "seeded16", "multicolor", "flat_nosmooth", "inverse"]
    recipes += [f"method{m}" for m in range(12)] + [f"differences{d}" for d in range(8)]
    for field, max_iter, bias in fields:
        for recipe in recipes:
            if field != "e30_160x90" and recipe.startswith(("method", "differences")):
                continue
            cases.append(dict(name=f"kfp_{recipe}_{field}", field=field, recipe=recipe, max_iter=max_iter,
                              field_bias=bias))
    return cases


# The mixed batch workload: field sizes and its zoom and cap ranges.
BATCH_SIZES = ((720, 480), (1280, 720), (1920, 1080), (3840, 2160))


def batch_centres() -> dict:
    """Centre pool per formula for the batch: seeded Misiurewicz points
    (Mandelbrot), the repelling fixed points of two seeded boundary
    constants (Julia), seeded preperiodic parameters (burning ship, tricorn);
    all with at least 120 digits, enough for 1e100."""
    c = centres()
    return {
        "mandelbrot": [dict(re=c[k]["re"], im=c[k]["im"]) for k in ("field_e100", "fhd_stack_e50",
                                                                   "field_640x360_e30")],
        "julia": [dict(re=c[k]["re"], im=c[k]["im"], julia=(c[k]["c_re"], c[k]["c_im"]))
                  for k in ("julia_fixed_1", "julia_fixed_2")],
        "burning-ship": [dict(re=c["burning_ship_deep"]["re"], im=c["burning_ship_deep"]["im"])],
        "tricorn": [dict(re=c["tricorn_deep"]["re"], im=c["tricorn_deep"]["im"])],
    }


def batch_mix(seed: int = 2024, count: int = 64, sizes=BATCH_SIZES, log_zoom=(10.0, 100.0),
              log_cap=(4.0, 6.0)) -> list[dict]:
    """A seeded mix of uneven fields: formula uniform over the four, centre
    from its pool, size from `sizes`, log10 zoom and log10 cap uniform over
    the given ranges."""
    import numpy as np

    rng = np.random.default_rng(seed)
    pool = batch_centres()
    formulas = ("mandelbrot", "julia", "burning-ship", "tricorn")
    mix = []
    for i in range(count):
        formula = formulas[int(rng.integers(0, 4))]
        centre = pool[formula][int(rng.integers(0, len(pool[formula])))]
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        mix.append(dict(name=f"batch{i:02d}_{formula}", formula=formula, re=centre["re"], im=centre["im"],
                        julia=centre.get("julia", ("0", "0")),
                        log10_zoom=float(rng.uniform(*log_zoom)), width=w, height=h,
                        max_iter=int(round(10.0 ** rng.uniform(*log_cap)))))
    return mix
