"""Generate the golden parity fixtures from the reference renderer itself.

The reference (renderer.cpp) is compiled by ``make -C oracle ref`` into
``oracle/_ref/mandelbrot.so`` with its release flags (no -march=native, hence
no compiler-chosen FMA: every double operation rounds on its own).  This
script runs every case of ``cases.py`` through that library's C ABI and
stores, per case, ``fixtures/<name>.npz`` with the float32 field, the uint32
iteration counts (escape index, cap for interior, 0 for NaN glitches) and,
for small cases, the six render planes.  Large cases store only SHA-256
digests and summary numbers in ``fixtures/index.json``.

Run here, where the reference sources exist:
    make -C oracle ref && python -m tests.golden.make_golden
"""

from __future__ import annotations

import ctypes
import json
import os
import sys

import numpy as np

from . import cases as case_defs
from .runner import _native, run_case, summary

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
FIXTURES = os.path.join(HERE, "fixtures")
REFERENCE_LIBRARY = os.path.join(ROOT, "oracle", "_ref", "mandelbrot.so")
REFERENCE_SOURCES = os.environ.get("REFERENCE_DIR", "/root/reference")


def _package_kfp():
    import importlib.util

    name = "fractal_audio_viz_gb300"
    if name not in sys.modules:
        package_dir = os.path.join(ROOT, "fractal-audio-viz_gb300")
        spec = importlib.util.spec_from_file_location(
            name, os.path.join(package_dir, "__init__.py"), submodule_search_locations=[package_dir])
        module = importlib.util.module_from_spec(spec)
        sys.modules[name] = module
        spec.loader.exec_module(module)
    return sys.modules[name].kfp


PLANE_LIMIT = 64 * 36  # store the f64 planes only for cases this small


def write_cases(library, cases, index) -> None:
    """Run `cases` through the reference build; store their fixtures and
    index entries."""
    for case in cases:
        result = run_case(library, case)
        info = summary(result)
        index["cases"][case["name"]] = info
        if case.get("store") != "hash":
            arrays = {"field": result["field"], "counts": result["counts"]}
            if case["width"] * case["height"] <= PLANE_LIMIT:
                for key in ("orbit_iteration", "phase", "de_x", "de_y", "test1", "test2"):
                    arrays[key] = result[key]
            np.savez_compressed(os.path.join(FIXTURES, case["name"] + ".npz"), **arrays)
        print(f"{case['name']:28s} sum={info['count_sum']:>12d} nan={info['nan_pixels']:>5d} "
              f"range=[{info['count_min']},{info['count_max']}]")


def main() -> int:
    native = _native()
    library = native.load(REFERENCE_LIBRARY)
    if "--deep-alternates" in sys.argv or "--deep-mandelbrot" in sys.argv:
        # Only the deep alternate-formula (or beyond-1e100 Mandelbrot)
        # fixtures, added to the index.
        path = os.path.join(FIXTURES, "index.json")
        with open(path, encoding="ascii") as handle:
            index = json.load(handle)
        cases = (case_defs.deep_alternate_cases() if "--deep-alternates" in sys.argv
                 else case_defs.deep_mandelbrot_cases())
        write_cases(library, cases, index)
        with open(path, "w", encoding="ascii") as handle:
            json.dump(index, handle, indent=1, sort_keys=True)
            handle.write("\n")
        return 0
    os.makedirs(FIXTURES, exist_ok=True)
    index = {"library": "oracle/_ref/mandelbrot.so (reference release build)", "cases": {}}
    all_cases = case_defs.parity_cases() + case_defs.alternate_cases()
    for case in all_cases:
        result = run_case(library, case)
        info = summary(result)
        index["cases"][case["name"]] = info
        if case.get("store") != "hash":
            arrays = {"field": result["field"], "counts": result["counts"]}
            if case["width"] * case["height"] <= PLANE_LIMIT:
                for key in ("orbit_iteration", "phase", "de_x", "de_y", "test1", "test2"):
                    arrays[key] = result[key]
            np.savez_compressed(os.path.join(FIXTURES, case["name"] + ".npz"), **arrays)
        print(f"{case['name']:28s} sum={info['count_sum']:>12d} nan={info['nan_pixels']:>5d} "
              f"range=[{info['count_min']},{info['count_max']}]")
    # KFP colour of stored fields through the reference's own transfer, with
    # the LUT built by the reference's Python (visualizer._kfp_palette_lut).
    sys.path.insert(0, REFERENCE_SOURCES)
    import visualizer  # noqa: E402  (reference pipeline, imported here only)

    package_kfp = _package_kfp()
    kfp_rgb = {}
    luts = {}
    for case in case_defs.kfp_cases():
        profile = package_kfp.recipe(case["recipe"])
        reference_profile = visualizer.KfpPalette(**{k: getattr(profile, k) for k in (
            "stops", "iter_div", "color_offset", "ratio", "color_method", "smooth_method", "smooth", "flat",
            "inverse_transition", "phase_color_strength", "multi_color", "blend_multi_color", "multi_colors",
            "power", "slopes", "slope_power", "slope_ratio", "slope_angle", "differences", "interior_color")})
        lut = np.asarray(visualizer._kfp_palette_lut(reference_profile), dtype=np.uint8)
        luts[case["recipe"]] = lut
        stored = np.load(os.path.join(FIXTURES, case["field"] + ".npz"))
        field_case = next(c for c in case_defs.parity_cases() if c["name"] == case["field"])
        options = visualizer.NativeKfpOptions.from_profile(reference_profile, field_bias=case["field_bias"])
        out = np.empty(stored["field"].size * 3, dtype=np.uint8)
        status = library.fractal_colourise_kfp(
            stored["field"].ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), field_case["width"], field_case["height"],
            case["max_iter"], 0.0, 0.0, 0.0, 0.5, ctypes.cast(ctypes.byref(options), ctypes.POINTER(native.KfpOptions)),
            lut.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), lut.shape[0], 0)
        assert status == 0, native.last_error(library)
        kfp_rgb[case["name"]] = out
        print(f"{case['name']:44s} mean={out.mean():7.2f}")
    np.savez_compressed(os.path.join(FIXTURES, "kfp_rgb.npz"), **kfp_rgb)
    np.savez_compressed(os.path.join(FIXTURES, "kfp_luts.npz"), **luts)
    with open(os.path.join(FIXTURES, "index.json"), "w", encoding="ascii") as handle:
        json.dump(index, handle, indent=1, sort_keys=True)
        handle.write("\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
