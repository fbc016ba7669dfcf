"""Run one parity case through any library exporting the renderer.h ABI.

The same call sequence drives the reference build (fixture generation), the
CPU oracle port and the GB300 library, so the three are compared on exactly
the same inputs.
"""

from __future__ import annotations

import hashlib

import numpy as np

from . import cases as case_defs


def _native():
    import importlib.util
    import os
    import sys

    name = "fractal_audio_viz_gb300.native"
    if name in sys.modules:
        return sys.modules[name]
    root = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    path = os.path.join(root, "fractal-audio-viz_gb300", "native.py")
    spec = importlib.util.spec_from_file_location(name, path)
    module = importlib.util.module_from_spec(spec)
    sys.modules[name] = module
    spec.loader.exec_module(module)
    return module


def options_for(case: dict):
    native = _native()
    return native.RenderOptions(**case.get("options", {}))


def run_case(library, case: dict, threads: int = 0) -> dict:
    """Execute ``case``; returns field (f32), counts (u32) and the planes."""
    native = _native()
    width, height = case["width"], case["height"]
    centre = case["centre"]
    x, y = centre["re"], centre["im"]
    zoom = case_defs.zoom_text(case["log10_zoom"]).encode("ascii")
    max_iter = case["max_iter"]
    options = options_for(case)
    formula = case["formula"]
    julia = case.get("julia", (0.0, 0.0))
    if case["kind"] == "direct":
        field, planes = native.render_fractal(
            library, width, height, zoom, x, y, max_iter, 256, False, threads=threads, formula=formula,
            julia=(float(julia[0]), float(julia[1])), options=options, planes=True)
    elif case["kind"] == "oneshot":
        bits = case_defs.precision_bits(x, y, case["log10_zoom"])
        field, planes = native.render_fractal(
            library, width, height, zoom, x, y, max_iter, bits, True, threads=threads, formula=formula,
            julia=(float(julia[0]), float(julia[1])), options=options, planes=True)
    else:
        root_log = case.get("root_log10_zoom", case["log10_zoom"])
        root_iter = case.get("root_max_iter", max_iter)
        bits = case_defs.precision_bits(x, y, root_log)
        root_zoom = case_defs.zoom_text(root_log).encode("ascii")
        creator_options = options if (formula != "mandelbrot" or case.get("options")) else None
        handle = native.create_reference(
            library, x, y, root_zoom, root_iter, bits, case["image_series_order"], formula=formula,
            julia=(str(julia[0]), str(julia[1])), options=creator_options, reusable=bool(case.get("clone")))
        handles = [handle]
        try:
            if case.get("clone"):
                handles.append(native.clone_reference(library, handle, zoom))
            field, planes = native.render_reference(
                library, handles[-1], width, height, zoom, max_iter, threads=threads,
                series_order=case["series_order"], series_block=case["series_block"], options=options,
                planes=True)
        finally:
            for h in reversed(handles):
                library.fractal_destroy_reference(h)
    counts = native.iteration_counts(field, planes["orbit_iteration"], max_iter)
    return {"field": field, "counts": counts, **planes}


def digest(array: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(array).tobytes()).hexdigest()


def summary(result: dict) -> dict:
    field, counts = result["field"], result["counts"]
    finite = np.isfinite(field)
    return {
        "field_sha256": digest(field),
        "counts_sha256": digest(counts),
        "count_sum": int(counts.astype(np.uint64).sum()),
        "nan_pixels": int((~finite).sum()),
        "count_min": int(counts.min()),
        "count_max": int(counts.max()),
    }
