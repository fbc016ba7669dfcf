"""GPU: the batched keyframe path against per-keyframe renders and the oracle.

fractal_gb300_render_keyframes_device renders many keyframes in a few
launches (a persistent lane-refill FP64 queue for the direct frames on a
second stream, a persistent floatexp queue or per-field plain launches for
the deep ones), optionally replayed as a CUDA graph and with autotuned launch
shapes.  None of that may change a pixel: every test here demands bit
equality with the single-keyframe entry points (whose parity with the
reference is tested in test_gpu_parity.py), and the direct queue's exact
shortcuts (squares reused, doubling by exponent, Brent cycle probe) are
checked against the oracle on interior-heavy whole-set views.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

from .golden import cases as case_defs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

WIDTH, HEIGHT = 192, 108
LEVELS = (0, 1, 3, 6, 9, 13, 14, 20, 31, 42, 54)


def _stack(package, product):
    levels = [lv for lv in case_defs.fhd_stack_levels() if lv[0] in LEVELS]
    e50 = case_defs.centres()["fhd_stack_e50"]
    return package.atlas.KeyframeStack(product, e50["re"], e50["im"], levels, step=math.log10(8.0))


def _buffers(n):
    fields = torch.full((n, WIDTH * HEIGHT), -1.0, dtype=torch.float32, device="cuda")
    counts = torch.zeros((n, WIDTH * HEIGHT), dtype=torch.int32, device="cuda")
    return fields, counts


def _bits(tensor):
    return tensor.cpu().numpy().view(np.uint32)


def _singles(stack, form):
    fields, counts = _buffers(len(stack.keyframes))
    for i, keyframe in enumerate(stack.keyframes):
        stack.render_device(keyframe, fields[i].data_ptr(), counts[i].data_ptr(), WIDTH, HEIGHT, form=form)
    torch.cuda.synchronize()
    return _bits(fields), _bits(counts)


def _batch(stack, form, **kw):
    fields, counts = _buffers(len(stack.keyframes))
    targets = [(fields[i].data_ptr(), counts[i].data_ptr()) for i in range(len(stack.keyframes))]
    stack.render_batch_device(targets, WIDTH, HEIGHT, form=form, **kw)
    torch.cuda.synchronize()
    return _bits(fields), _bits(counts)


@pytest.mark.parametrize("form", [0, 1])
def test_batch_equals_single_keyframe_renders(package, product, form):
    stack = _stack(package, product)
    try:
        want_field, want_counts = _singles(stack, form)
        got_field, got_counts = _batch(stack, form)
        direct = np.array([k.reference is None for k in stack.keyframes])
    finally:
        stack.close()
    # In form 1 the direct levels that shallow_perturbation() admits render
    # from the root reference in the floatexp form's shallow mode, in the
    # batch and alone alike; the others stay on the FP64 direct path, where
    # the batch takes the smooth value's logarithms in FP32 (counts equal,
    # smooth values within a few float ulps).
    assert direct.any() and any(k.shallow_reference is not None for k in stack.keyframes)
    np.testing.assert_array_equal(got_counts, want_counts)
    if form == 0:
        np.testing.assert_array_equal(got_field, want_field)
        return
    fp64 = np.array([k.reference is None and k.shallow_reference is None for k in stack.keyframes])
    np.testing.assert_array_equal(got_field[~fp64], want_field[~fp64])
    got = got_field[fp64].view(np.float32).astype(np.float64)
    want = want_field[fp64].view(np.float32).astype(np.float64)
    assert np.all(np.abs(got - want) <= 4e-6 * np.maximum(1.0, np.abs(want))), np.max(np.abs(got - want))


def test_batch_graph_replay_order_and_autotune_keep_pixels(package, product):
    stack = _stack(package, product)
    try:
        want_field, want_counts = _batch(stack, 1)
        reverse = list(range(len(stack.keyframes)))[::-1]
        runs = [
            _batch(stack, 1, graph=True),
            _batch(stack, 1, graph=True),          # replay of the cached graph
            _batch(stack, 1, order=reverse),
            _batch(stack, 1, autotune=True),
            _batch(stack, 0, graph=True),
        ]
        shapes = stack.queue_shapes()
    finally:
        stack.close()
    for field, counts in runs[:4]:
        np.testing.assert_array_equal(counts, want_counts)
        np.testing.assert_array_equal(field, want_field)
    assert shapes[0] > 0 and shapes[2] > 0 and shapes[1] >= 0 and shapes[3] >= 0
    # The plain form differs from floatexp only within the floatexp budget.
    plain_counts = runs[4][1]
    assert np.count_nonzero(plain_counts != want_counts) <= 1e-4 * want_counts.size + 2


@pytest.mark.parametrize("view", [
    ("whole_set", "-0.5", "0.0", "1", 320, 180, 3000),
    ("seahorse", "-0.7436", "0.1318", "180", 256, 144, 6000),
    ("bulbs", "-1.25", "0.0", "6", 200, 120, 5000),
])
def test_direct_queue_matches_oracle_on_interior_views(package, product, oracle_port, view):
    """Interior-heavy direct views, where the cycle probe settles most
    interior pixels early: counts and field bits equal the oracle's."""
    native = package.native
    _, x, y, zoom, w, h, cap = view
    got = native.render_fractal(product, w, h, zoom.encode(), x, y, cap, 256, False, threads=0)
    want = native.render_fractal(oracle_port, w, h, zoom.encode(), x, y, cap, 256, False, threads=0)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_direct_queue_device_entry_on_two_streams(package, product):
    """Back-to-back device calls on different caller streams share the
    thread's scratch; the library orders them, so both results are exact."""
    import ctypes

    native = package.native
    fields, counts = _buffers(2)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    zooms = [b"1", b"40"]
    options = native.RenderOptions()
    for i in range(2):
        status = product.fractal_gb300_render_direct_device(
            ctypes.c_void_p(fields[i].data_ptr()), ctypes.c_void_p(counts[i].data_ptr()), WIDTH, HEIGHT, zooms[i],
            b"-0.5", b"0.0", 2000, 0, 0.0, 0.0, ctypes.byref(options), ctypes.c_void_p(streams[i].cuda_stream))
        assert status == 0, native.last_error(product)
    torch.cuda.synchronize()
    for i in range(2):
        want = native.render_fractal(product, WIDTH, HEIGHT, zooms[i], "-0.5", "0.0", 2000, 256, False)
        np.testing.assert_array_equal(_bits(fields[i]), want.view(np.uint32))


def test_tile_queue_static_and_learned_orders_keep_pixels(package, product):
    """The tile-scheduled floatexp queue (static order, probe, and the order
    a cost network predicts) renders exactly the pixels of the pixel-chunk
    queue, and reports per-tile costs and its makespan/tail."""
    import ctypes

    native = package.native
    stack = _stack(package, product)
    net = product.fractal_gb300_costnet_create(3)
    assert net, native.last_error(product)
    try:
        want_field, want_counts = _batch(stack, 1)
        static = _batch(stack, 1, tiles=native.BATCH_TILES | native.BATCH_PROBE)
        count = ctypes.c_int(0)
        timing = (ctypes.c_double * 2)()
        queued = [k for k in stack.keyframes if k.reference is not None or k.shallow_reference is not None]
        tiles_expected = len(queued) * ((WIDTH + 63) // 64) * ((HEIGHT + 63) // 64)
        cost = np.zeros(tiles_expected, dtype=np.float32)
        features = np.zeros((tiles_expected, 320), dtype=np.uint16)
        assert product.fractal_gb300_last_tiles(ctypes.byref(count), cost.ctypes.data, features.ctypes.data,
                                                tiles_expected, timing) == 0, native.last_error(product)
        assert count.value == tiles_expected
        assert np.all(cost > 0)
        assert timing[0] > 0 and 0 <= timing[1] <= timing[0]
        probe = (features[:, :256].astype(np.uint32) << 16).view(np.float32)
        assert np.all((probe >= 0) & (probe <= 1.0))
        assert product.fractal_gb300_set_cost_network(net) == 0
        learned = _batch(stack, 1, tiles=native.BATCH_LEARNED | native.BATCH_TILES)
        learned_graph = _batch(stack, 1, tiles=native.BATCH_LEARNED | native.BATCH_TILES, graph=True)
    finally:
        product.fractal_gb300_set_cost_network(None)
        product.fractal_gb300_costnet_destroy(net)
        stack.close()
    for field, counts in (static, learned, learned_graph):
        np.testing.assert_array_equal(counts, want_counts)
        np.testing.assert_array_equal(field, want_field)


def test_mixed_formula_batch_matches_fixtures_and_singles(package, product):
    """A batch of uneven fields: Julia, burning ship and tricorn deep views
    (plain form launches in both forms), a Mandelbrot deep view (floatexp
    queue in form 1) and shallow alternate views (direct queue grouped by
    formula).  Every frame equals its single-call render; the alternate ones
    also equal the reference's own fixtures."""
    import ctypes

    from .conftest import golden_arrays

    native = package.native
    wanted = ["julia_fixed_1_e9_96x54", "julia_fixed_2_e15_64x36", "burning-ship_e7_96x54", "tricorn_e12_64x36"]
    cases = [c for c in case_defs.alternate_cases() if c["name"] in wanted]
    e30 = case_defs.centres()["field_640x360_e30"]
    cases.append(case_defs._m("mandel_e30", kind="reference", centre=e30, log10_zoom=30.0, width=80, height=45,
                              max_iter=50_000))
    handles, frames_meta = [], []
    try:
        for case in cases:
            bits = case_defs.precision_bits(case["centre"]["re"], case["centre"]["im"], case["log10_zoom"])
            handle = native.create_reference(product, case["centre"]["re"], case["centre"]["im"],
                                             case_defs.zoom_text(case["log10_zoom"]).encode(), case["max_iter"],
                                             bits, case["image_series_order"], formula=case["formula"],
                                             julia=case.get("julia", ("0", "0")))
            assert handle, native.last_error(product)
            handles.append(handle)
            frames_meta.append((case, handle, case_defs.zoom_text(case["log10_zoom"]).encode()))
        # Shallow views of two alternate references (direct path, by formula).
        for case, handle, _ in frames_meta[:1] + frames_meta[2:3]:
            frames_meta.append((dict(case, name=case["name"] + "_shallow", log10_zoom=3.0), handle, b"1000"))
        for form in (0, 1):
            bufs = []
            frames = (native.Keyframe * len(frames_meta))()
            for i, (case, handle, zoom) in enumerate(frames_meta):
                w, h = case["width"], case["height"]
                field = torch.full((w * h,), -1.0, dtype=torch.float32, device="cuda")
                counts = torch.zeros((w * h,), dtype=torch.int32, device="cuda")
                bufs.append((field, counts))
                frames[i].field = field.data_ptr()
                frames[i].counts = counts.data_ptr()
                frames[i].zoom_text = zoom
                frames[i].reference = handle
                frames[i].max_iter = case["max_iter"]
            # One size per batch call: group by size.
            sizes = sorted({(c["width"], c["height"]) for c, _, _ in frames_meta})
            for w, h in sizes:
                idx = [i for i, (c, _, _) in enumerate(frames_meta) if (c["width"], c["height"]) == (w, h)]
                sub = (native.Keyframe * len(idx))(*[frames[i] for i in idx])
                options = native.RenderOptions()
                status = product.fractal_gb300_render_keyframes_device(sub, len(idx), w, h, None, None, 3, 256,
                                                                       ctypes.byref(options), form, 1, None)
                assert status == 0, native.last_error(product)
            torch.cuda.synchronize()
            for (case, handle, zoom), (field, counts) in zip(frames_meta, bufs):
                w, h = case["width"], case["height"]
                single_f = torch.full((w * h,), -1.0, dtype=torch.float32, device="cuda")
                single_c = torch.zeros((w * h,), dtype=torch.int32, device="cuda")
                options = native.RenderOptions()
                status = product.fractal_gb300_render_reference_device(
                    ctypes.c_void_p(single_f.data_ptr()), ctypes.c_void_p(single_c.data_ptr()), w, h, zoom,
                    ctypes.c_void_p(handle), case["max_iter"], 3, 256, ctypes.byref(options), form, None)
                assert status == 0, native.last_error(product)
                torch.cuda.synchronize()
                np.testing.assert_array_equal(counts.cpu().numpy(), single_c.cpu().numpy(), err_msg=case["name"])
                if form == 1 and case["name"].endswith("_shallow"):
                    # The floatexp form's batch takes direct frames' smooth
                    # logarithms in FP32 (a few float ulps).
                    got, want = field.cpu().numpy(), single_f.cpu().numpy()
                    assert np.all(np.abs(got - want) <= 4e-6 * np.maximum(1.0, np.abs(want))), case["name"]
                else:
                    np.testing.assert_array_equal(_bits(field), _bits(single_f), err_msg=case["name"])
                stored = golden_arrays(case["name"]) if case["formula"] != "mandelbrot" else None
                if stored is not None and not case["name"].endswith("_shallow"):
                    got = counts.cpu().numpy().view(np.uint32)
                    want = stored["counts"].copy()
                    if case["formula"] == "julia":
                        # Fixture counts are orbit_iteration + 1, and the
                        # reference's Julia orbit_iteration is the escape
                        # index itself (not index - 1 as for the parameter
                        # plane): the escape index is one less.
                        escaped = (want > 0) & (want < case["max_iter"])
                        want[escaped] -= 1
                    np.testing.assert_array_equal(got, want, err_msg=case["name"])
    finally:
        for handle in handles:
            product.fractal_destroy_reference(handle)
