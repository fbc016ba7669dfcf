"""Batches of uneven fields of every formula through one device call.

``FieldSet`` prepares one reference handle per field (its own centre, zoom,
cap and formula, as the reference pipeline's ``_create_native_reference``
does for each field, visualizer.py:6250-6346) and renders all of them through
``fractal_gb300_render_fields_device``: in the floatexp form the
Mandelbrot fields (and, on request, the other formulas') in one persistent
FP32 queue beside the FP64 launches of the rest; the FP64 plain form
otherwise.  Fields below 1e12 carry the
shallow flag, so the plain form renders them on the direct path as the
reference pipeline does (visualizer.py:6152).
"""

from __future__ import annotations

import ctypes
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import Optional

from . import atlas, native

SHALLOW_LOG10_ZOOM = 12.0


@dataclass
class FieldSpec:
    formula: str            # "mandelbrot", "julia", "burning-ship", "tricorn"
    x: str                  # centre, decimal strings
    y: str
    log10_zoom: float
    width: int
    height: int
    max_iter: int
    julia: tuple[str, str] = ("0", "0")


class FieldSet:
    """Reference handles for a list of fields and their batched render."""

    def __init__(self, library, specs: list[FieldSpec], *, image_series_order: int = 32, threads: int = 8,
                 initializer=None):
        self.library = library
        self.specs = list(specs)
        self.zooms = [atlas.zoom_text(s.log10_zoom) for s in self.specs]

        def create(i: int) -> int:
            s = self.specs[i]
            bits = atlas.precision_bits(s.x, s.y, s.log10_zoom)
            return native.create_reference(library, s.x, s.y, self.zooms[i], s.max_iter, bits, image_series_order,
                                           formula=s.formula, julia=s.julia)

        # Reference creation (MPFR orbit, series) is host work per field;
        # the library's registry takes concurrent creators.  `initializer`
        # runs in each worker thread first (e.g. to make the caller's CUDA
        # device current there: a new thread starts on device 0).
        with ThreadPoolExecutor(max(1, threads), initializer=initializer) as pool:
            self.handles = list(pool.map(create, range(len(self.specs))))

    def frames(self, targets):
        """FractalGb300Field array for `targets`: per field (field_ptr,
        counts_ptr, de_x_ptr, de_y_ptr), the last three may be None."""
        frames = (native.Field * len(self.specs))()
        for i, (spec, target) in enumerate(zip(self.specs, targets)):
            field_ptr, counts_ptr, de_x, de_y = target
            frames[i].field = field_ptr
            frames[i].counts = counts_ptr
            frames[i].de_x = de_x
            frames[i].de_y = de_y
            frames[i].zoom_text = self.zooms[i]
            frames[i].reference = self.handles[i]
            frames[i].width = spec.width
            frames[i].height = spec.height
            frames[i].max_iter = spec.max_iter
            frames[i].flags = native.KEYFRAME_SHALLOW if spec.log10_zoom < SHALLOW_LOG10_ZOOM else 0
        return frames

    def render_device(self, targets, *, form: int, stream: int = 0, graph: bool = False, autotune: bool = False,
                      tiles: int = 0, fp32_alternates: bool = False, series_order: int = 3, series_block: int = 256,
                      options: Optional[native.RenderOptions] = None) -> None:
        """Enqueue every field in one batched call (GB300 extension ABI).
        `fp32_alternates` puts the other formulas' fields in the FP32 queue
        too (faster, but their counts drift from the FP64 form's)."""
        options = options or native.RenderOptions()
        frames = self.frames(targets)
        flags = ((native.BATCH_GRAPH if graph else 0) | (native.BATCH_AUTOTUNE if autotune else 0) | tiles
                 | (native.BATCH_FP32_ALTERNATES if fp32_alternates else 0))
        status = self.library.fractal_gb300_render_fields_device(
            frames, len(self.specs), None, None, series_order, series_block, ctypes.byref(options), form, flags,
            ctypes.c_void_p(stream))
        if status != 0:
            raise native.NativeError(native.last_error(self.library))

    def close(self) -> None:
        for handle in self.handles:
            self.library.fractal_destroy_reference(handle)
        self.handles = []
