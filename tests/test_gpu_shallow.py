"""GPU: the floatexp form's shallow mode against the FP64 direct path.

Below 1e12 the reference pipeline renders a field by direct FP64 iteration
(visualizer.py:6152, renderer.cpp:9838-10562).  The floatexp form renders
those fields by plain FP32 perturbation against the stack's root reference
orbit, from iteration 0 with unlimited rebasing (FxParams::shallow).  Its
counts may differ from the FP64 form only where rounding decides an escape
iteration; the floatexp form's budget is 1e-4 of pixels,
the tolerance used here (plus two pixels of slack per field set).
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

from .golden import cases as case_defs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MISMATCH_BUDGET = 1e-4


def _render_stack(stack, width, height, form):
    n = len(stack.keyframes)
    fields = torch.full((n, width * height), -1.0, dtype=torch.float32, device="cuda")
    counts = torch.zeros((n, width * height), dtype=torch.int32, device="cuda")
    targets = [(fields[i].data_ptr(), counts[i].data_ptr()) for i in range(n)]
    stack.render_batch_device(targets, width, height, form=form)
    torch.cuda.synchronize()
    return fields.cpu().numpy(), counts.cpu().numpy()


def test_shallow_levels_match_the_fp64_direct_form(package, product):
    """The direct levels of the FHD stack that the floatexp form renders in
    its shallow mode (plus one deep level so that the stack has its root
    reference) at 320x180: counts within the budget, smooth values close
    where the counts agree, no NaN."""
    e50 = case_defs.centres()["fhd_stack_e50"]
    levels = [lv for lv in case_defs.fhd_stack_levels() if lv[0] <= 14]
    stack = package.atlas.KeyframeStack(product, e50["re"], e50["im"], levels, step=math.log10(8.0))
    try:
        shallow = [i for i, k in enumerate(stack.keyframes) if k.shallow_reference is not None]
        direct = [i for i, k in enumerate(stack.keyframes) if k.reference is None]
        # Level 0 reaches the main cardioid, 12-13 are at 1e10 and deeper:
        # those keep the FP64 direct iteration.
        assert len(direct) == 14 and shallow == [i for i in direct if 1 <= stack.keyframes[i].level <= 11]
        plain_field, plain_counts = _render_stack(stack, 320, 180, 0)
        fe_field, fe_counts = _render_stack(stack, 320, 180, 1)
    finally:
        stack.close()
    plain_counts, fe_counts = plain_counts[shallow], fe_counts[shallow]
    plain_field, fe_field = plain_field[shallow], fe_field[shallow]
    assert not np.isnan(fe_field).any()
    differ = plain_counts != fe_counts
    per_level = differ.sum(axis=1)
    assert differ.sum() <= MISMATCH_BUDGET * differ.size + 2, per_level
    same = ~differ
    error = np.abs(fe_field[same].astype(np.float64) - plain_field[same].astype(np.float64))
    assert np.median(error) <= 1e-5
    assert np.quantile(error, 0.99) <= 2e-3, np.quantile(error, 0.99)


@pytest.mark.parametrize("view", [
    ("whole_set", "-0.5", "0.0", 0.0, 320, 180, 3000),
    ("bulbs", "-1.25", "0.0", math.log10(6.0), 200, 120, 5000),
    ("antenna_minibrot", "-1.7549", "0.0", math.log10(50.0), 256, 144, 6000),
])
def test_shallow_mode_on_interior_views(package, product, oracle_port, view):
    """Interior-heavy views rendered from a reference at the view centre in
    the shallow mode against the oracle's direct FP64 render: the cardioid /
    bulb cull and the rebasing keep interior pixels at the cap.  The first
    two views reach the main cardioid or the period-2 bulb, whose parabolic
    boundary points make counts sensitive to a 1e-4-pixel error in c (the
    atlas keeps the FP64 direct iteration for such views,
    atlas.view_meets_interior; the seahorse valley between them differs on 5
    % of its pixels), so the bound here is 5e-3; the third, a minibrot on the
    antenna, is a view the rule admits."""
    native = package.native
    _, x, y, log_zoom, w, h, cap = view
    zoom = native.zoom_text(log_zoom)
    handle = native.create_reference(product, x, y, zoom, cap, 256, 32, reusable=True)
    field = torch.empty(w * h, dtype=torch.float32, device="cuda")
    counts = torch.empty(w * h, dtype=torch.int32, device="cuda")
    try:
        options = native.RenderOptions()
        status = product.fractal_gb300_render_reference_device(
            ctypes.c_void_p(field.data_ptr()), ctypes.c_void_p(counts.data_ptr()), w, h, zoom,
            ctypes.c_void_p(handle), cap, 3, 256, ctypes.byref(options), 1, None)
        assert status == 0, native.last_error(product)
        torch.cuda.synchronize()
    finally:
        product.fractal_destroy_reference(handle)
    got, got_counts = field.cpu().numpy(), counts.cpu().numpy().astype(np.uint32)
    want, planes = native.render_fractal(oracle_port, w, h, zoom, x, y, cap, 256, False, threads=0, planes=True)
    want_counts = native.iteration_counts(want, planes["orbit_iteration"], cap)
    assert not np.isnan(got).any()
    interior = want_counts == cap
    assert interior.sum() > 0.05 * want.size
    differ = got_counts != want_counts
    report = (int(differ.sum()), int((differ & interior).sum()), int(interior.sum()), want.size)
    assert differ.sum() <= 5e-3 * want.size, report
    # FP64-interior pixels stay interior, bar the few on the parabolic
    # boundaries that escape after many iterations at FP32 precision.
    assert (differ & interior).sum() <= 1e-3 * interior.sum() + 2, report


def test_shallow_flag_in_form0_takes_the_direct_path(package, product):
    """Form 0 ignores the handle of a shallow frame: the pixels are the direct
    FP64 path's, bit for bit."""
    native = package.native
    e50 = case_defs.centres()["fhd_stack_e50"]
    levels = [lv for lv in case_defs.fhd_stack_levels() if lv[0] in (3, 9, 14)]
    stack = package.atlas.KeyframeStack(product, e50["re"], e50["im"], levels, step=math.log10(8.0))
    try:
        w, h = 192, 108
        field, counts = _render_stack(stack, w, h, 0)
        for i, keyframe in enumerate(stack.keyframes):
            if keyframe.reference is not None:
                continue
            want = native.render_fractal(product, w, h, native.zoom_text(keyframe.log10_zoom), e50["re"],
                                         e50["im"], keyframe.max_iter, 256, False, threads=0)
            np.testing.assert_array_equal(field[i].view(np.uint32), want.view(np.uint32))
    finally:
        stack.close()
    field = torch.empty(w * h, dtype=torch.float32, device="cuda")
    frames = (native.Keyframe * 1)()
    frames[0].field = field.data_ptr()
    frames[0].zoom_text = b"1"
    frames[0].max_iter = 100
    frames[0].flags = 2
    assert product.fractal_gb300_render_keyframes_device(frames, 1, w, h, b"0", b"0", 3, 256, None, 1, 0,
                                                        None) != 0
    assert "flags" in native.last_error(product)
