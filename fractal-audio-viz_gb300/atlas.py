"""Atlas-keyframe orchestration around the native field renderer.

Host-side mirror of the reference pipeline's helpers that decide what the
renderer is asked to do for an atlas of keyframes (visualizer.py):

* ``max_iterations``         iteration cap per depth        (:6958-6979)
* ``atlas_geometry``         logarithmic keyframe ladder    (:7628-7661)
* ``reference_tier_logs``    BLA input-radius tiers         (:6409-6481)
* ``select_reference``       tier used by one keyframe      (:6484-6510)
* ``precision_bits``         MPFR precision of a reference  (:5003-5036)
* ``zoom_text``              decimal zoom string            (:5118-5124)

``KeyframeStack`` prepares the shared MPFR reference and its tier clones on
a library and renders every keyframe, shallow ones through the direct path
(below 1e12, visualizer.py:6152) and deep ones from the selected tier.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Optional

from . import native


def max_iterations(log10_zoom: float, base: int, per_decade: int, cap: int) -> int:
    return min(cap, max(64, int(base + per_decade * max(0.0, log10_zoom))))


def atlas_geometry(zooms, keyframe_factor: float) -> tuple[float, float, int]:
    step = math.log10(max(1.05, keyframe_factor))
    minimum = float(min(zooms))
    maximum = float(max(zooms))
    origin = math.floor(minimum / step) * step
    count = max(0, int(math.ceil((maximum - origin) / step - 1.0e-12)))
    return origin, step, count


def reference_tier_logs(max_log_zoom: float, atlas_step: Optional[float] = None) -> list[float]:
    maximum = float(max_log_zoom)
    if not math.isfinite(maximum) or maximum < 12.0:
        return []
    starts = [12.0]
    if maximum <= 24.0:
        return starts
    decades = [float(v) for v in range(20, int(maximum) + 1, 10)]
    if atlas_step is not None:
        step = float(atlas_step)
        decades = [max(12.0, math.floor(v / step) * step - 3.0 * step) for v in decades]
    starts.extend(decades)
    starts = sorted(set(starts))
    if maximum > starts[-1] + 1.0e-9:
        starts.append(maximum)
    return sorted(set(starts))


def select_reference(references: list, log_zoom: float, minimum_margin_log: float = 0.0):
    margin = max(0.0, float(minimum_margin_log))
    selected = None
    for start_log, reference in references:
        if start_log <= 12.0 + 1.0e-9:
            if float(log_zoom) + 1.0e-9 < start_log:
                break
        elif margin > 0.0:
            if float(log_zoom) <= start_log + margin + 1.0e-9:
                break
        elif float(log_zoom) + 1.0e-9 < start_log:
            break
        selected = reference
    return selected


def _fractional_places(text: str) -> int:
    text = text.strip().lstrip("+-")
    return len(text.split(".", 1)[1]) if "." in text else 0


def precision_bits(x_center: str, y_center: str, log10_zoom: float) -> int:
    digits = max(50, 32 + int(math.ceil(max(0.0, log10_zoom))), _fractional_places(x_center),
                 _fractional_places(y_center))
    return max(256, int(digits * math.log2(10.0)) + 32)


def zoom_text(log10_zoom: float) -> bytes:
    return native.zoom_text(log10_zoom)


# Zoom (log10) from which a direct-path level keeps the FP64 direct
# iteration in the floatexp form: there FP64's 2^-53 resolution leaves fewer
# than about ten bits below a 1080-row pixel, so the FP64 counts are decided
# by FP64 rounding and only FP64 reproduces them.
SHALLOW_FP64_LOG10_ZOOM = 10.0


def view_meets_interior(x: float, y: float, log10_zoom: float, aspect: float = 16.0 / 9.0) -> bool:
    """Whether a view reaches the main cardioid's or period-2 bulb's bounding
    box (0.05 margin), as the direct path's interior test decides it.  Near
    those boundaries escape times grow without bound (parabolic points), so a
    1e-4-pixel error in c moves many counts: such views keep the FP64 direct
    iteration in the floatexp form."""
    half_h = 0.5 * 2.8 / 10.0 ** log10_zoom + 0.05
    half_w = 0.5 * 2.8 * aspect / 10.0 ** log10_zoom + 0.05
    cardioid = x + half_w >= -0.80 and x - half_w <= 0.40 and y + half_h >= -0.70 and y - half_h <= 0.70
    bulb = x + half_w >= -1.30 and x - half_w <= -0.70 and y + half_h >= -0.30 and y - half_h <= 0.30
    return cardioid or bulb


def shallow_perturbation(x: str, y: str, log10_zoom: float) -> bool:
    """Whether the floatexp form renders a direct-path level (below 1e12) by
    FP32 perturbation from the root reference (its shallow mode) rather than
    by the FP64 direct iteration."""
    if log10_zoom >= SHALLOW_FP64_LOG10_ZOOM:
        return False
    return not view_meets_interior(float(x), float(y), log10_zoom)


@dataclass
class Keyframe:
    level: int
    log10_zoom: float
    max_iter: int
    reference: Optional[int]  # handle for deep levels, None for direct ones
    # Direct levels of a stack that has a root reference, where
    # shallow_perturbation() holds: that handle, which the floatexp form
    # (form 1) renders them from in its shallow mode.
    shallow_reference: Optional[int] = None


class KeyframeStack:
    """A ladder of keyframes over one centre with shared reference tiers.

    ``levels`` are (level, log10 zoom, cap).  The root reference is made once
    at the deepest level with the largest cap; each tier is a clone that
    rebuilds only the radius-dependent tables (visualizer.py:6250-6481).
    """

    def __init__(self, library, x_center: str, y_center: str, levels, *, step: float,
                 image_series_order: int = 32):
        self.library = library
        self.x = x_center
        self.y = y_center
        self.handles: list[int] = []
        deepest = max(log_zoom for _, log_zoom, _ in levels)
        cap = max(max_iter for _, _, max_iter in levels)
        tiers = reference_tier_logs(deepest, step)
        references = []
        if tiers:
            bits = precision_bits(x_center, y_center, deepest)
            root = native.create_reference(library, x_center, y_center, zoom_text(deepest), cap, bits,
                                           image_series_order, reusable=True)
            self.handles.append(root)
            for tier in tiers:
                clone = native.clone_reference(library, root, zoom_text(tier))
                self.handles.append(clone)
                references.append((tier, clone))
        self.keyframes = []
        root = self.handles[0] if self.handles else None
        for level, log_zoom, max_iter in levels:
            reference = select_reference(references, log_zoom) if log_zoom >= 12.0 else None
            shallow = root if reference is None and shallow_perturbation(x_center, y_center, log_zoom) else None
            self.keyframes.append(Keyframe(level, log_zoom, max_iter, reference, shallow))

    def close(self) -> None:
        for handle in reversed(self.handles):
            self.library.fractal_destroy_reference(handle)
        self.handles.clear()

    def render_device(self, keyframe: Keyframe, field_ptr: int, counts_ptr: int, width: int, height: int,
                      *, form: int = 0, series_order: int = 3, series_block: int = 256,
                      options: Optional[native.RenderOptions] = None, stream: int = 0) -> None:
        """Enqueue one keyframe into device buffers (GB300 extension ABI).

        Direct levels take the FP64 direct path in form 0; in form 1 they
        render from the root reference in the floatexp form's shallow mode
        when the stack has one."""
        options = options or native.RenderOptions()
        zoom = zoom_text(keyframe.log10_zoom)
        if keyframe.reference is None and form == 1 and keyframe.shallow_reference is not None:
            status = self.library.fractal_gb300_render_reference_device(
                ctypes.c_void_p(field_ptr), ctypes.c_void_p(counts_ptr), width, height, zoom,
                ctypes.c_void_p(keyframe.shallow_reference), keyframe.max_iter, series_order, series_block,
                ctypes.byref(options), form, ctypes.c_void_p(stream))
        elif keyframe.reference is None:
            status = self.library.fractal_gb300_render_direct_device(
                ctypes.c_void_p(field_ptr), ctypes.c_void_p(counts_ptr), width, height, zoom,
                self.x.encode("ascii"), self.y.encode("ascii"), keyframe.max_iter, 0, 0.0, 0.0,
                ctypes.byref(options), ctypes.c_void_p(stream))
        else:
            status = self.library.fractal_gb300_render_reference_device(
                ctypes.c_void_p(field_ptr), ctypes.c_void_p(counts_ptr), width, height, zoom,
                ctypes.c_void_p(keyframe.reference), keyframe.max_iter, series_order, series_block,
                ctypes.byref(options), form, ctypes.c_void_p(stream))
        if status != 0:
            raise native.NativeError(native.last_error(self.library))

    def render_batch_device(self, targets, width: int, height: int, *, form: int = 0, series_order: int = 3,
                            series_block: int = 256, options: Optional[native.RenderOptions] = None,
                            stream: int = 0, graph: bool = False, autotune: bool = False, order=None,
                            tiles: int = 0) -> None:
        """Enqueue every keyframe in one batched call (GB300 extension ABI).

        ``targets`` holds one (field_ptr, counts_ptr) pair per keyframe;
        ``order`` optionally lists keyframe indices in claim order (costliest
        first).  Results equal per-keyframe ``render_device`` calls.
        """
        options = options or native.RenderOptions()
        indices = list(order) if order is not None else list(range(len(self.keyframes)))
        frames = (native.Keyframe * len(indices))()
        zooms = []
        for slot, index in enumerate(indices):
            keyframe = self.keyframes[index]
            field_ptr, counts_ptr = targets[index]
            zooms.append(zoom_text(keyframe.log10_zoom))
            frames[slot].field = field_ptr
            frames[slot].counts = counts_ptr
            frames[slot].zoom_text = zooms[-1]
            if keyframe.reference is None and keyframe.shallow_reference is not None:
                frames[slot].reference = keyframe.shallow_reference
                frames[slot].flags = native.KEYFRAME_SHALLOW
            else:
                frames[slot].reference = keyframe.reference
            frames[slot].max_iter = keyframe.max_iter
        flags = (native.BATCH_GRAPH if graph else 0) | (native.BATCH_AUTOTUNE if autotune else 0) | tiles
        status = self.library.fractal_gb300_render_keyframes_device(
            frames, len(indices), width, height, self.x.encode("ascii"), self.y.encode("ascii"), series_order,
            series_block, ctypes.byref(options), form, flags, ctypes.c_void_p(stream))
        if status != 0:
            raise native.NativeError(native.last_error(self.library))

    def queue_shapes(self) -> list[int]:
        values = (ctypes.c_int * 4)()
        if self.library.fractal_gb300_queue_shapes(values, 4) != 0:
            raise native.NativeError(native.last_error(self.library))
        return list(values)

    def render_host(self, keyframe: Keyframe, width: int, height: int, *, threads: int = 0,
                    series_order: int = 3, series_block: int = 256, planes: bool = False,
                    options: Optional[native.RenderOptions] = None):
        """Render one keyframe through the renderer.h ABI into host memory.

        With the CUDA backend's floatexp form (options.backend 4) a direct
        level renders from the root reference in the shallow mode."""
        zoom = zoom_text(keyframe.log10_zoom)
        shallow = (keyframe.reference is None and keyframe.shallow_reference is not None
                   and options is not None and options.backend == native.BACKEND_CUDA)
        if shallow:
            return native.render_reference(self.library, keyframe.shallow_reference, width, height, zoom,
                                           keyframe.max_iter, threads=threads, series_order=series_order,
                                           series_block=series_block, options=options, planes=planes)
        if keyframe.reference is None:
            return native.render_fractal(self.library, width, height, zoom, self.x, self.y, keyframe.max_iter,
                                         256, False, threads=threads, options=options, planes=planes)
        return native.render_reference(self.library, keyframe.reference, width, height, zoom,
                                       keyframe.max_iter, threads=threads, series_order=series_order,
                                       series_block=series_block, options=options, planes=planes)
