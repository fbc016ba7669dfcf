"""GPU: the tile-cost network's tensor-core kernels against the CPU oracle.

The tcgen05 GEMM (BF16 operands through TMA, FP32 accumulator in TMEM) is
compared with a float64 product of the same BF16 values; the network's
forward pass and every gradient of one training step are compared with
oracle/costnet.py, which rounds to BF16 at the same points.
"""

from __future__ import annotations

import ctypes
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import costnet as oracle  # noqa: E402


def _bf16(array):
    return torch.from_numpy(oracle.to_bf16_bits(array)).view(torch.bfloat16).cuda()


@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (256, 16, 128), (128, 64, 320), (384, 272, 1024)])
def test_tensor_core_gemm_matches_float64(product, m, n, k):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    a = oracle.round_bf16(rng.standard_normal((m, k)).astype(np.float32))
    b = oracle.round_bf16(rng.standard_normal((n, k)).astype(np.float32))
    b_rows = (n + 255) // 256 * 256
    b_padded = np.zeros((b_rows, k), dtype=np.float32)
    b_padded[:n] = b
    a_dev = _bf16(a)
    b_dev = _bf16(b_padded)
    c_dev = torch.full((m, n), float("nan"), dtype=torch.float32, device="cuda")
    status = product.fractal_gb300_gemm_bf16(a_dev.data_ptr(), b_dev.data_ptr(), c_dev.data_ptr(), m, n, k, b_rows,
                                             None)
    assert status == 0, product.fractal_last_error()
    got = c_dev.cpu().numpy().astype(np.float64)
    want = a.astype(np.float64) @ b.astype(np.float64).T
    # FP32 accumulation of k products of BF16 values.
    scale = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64).T
    assert np.all(np.abs(got - want) <= 1e-6 * scale + 1e-6), np.max(np.abs(got - want) / (scale + 1e-6))


def test_tensor_core_gemm_rejects_bad_shapes(product):
    status = product.fractal_gb300_gemm_bf16(None, None, None, 100, 16, 64, 256, None)
    assert status == 1


def _features(rng, rows):
    x = np.zeros((rows, oracle.FEATURES), dtype=np.float32)
    x[:, :256] = rng.random((rows, 256))
    x[:, 256] = rng.random(rows)
    x[:, 257] = rng.random(rows)
    return oracle.round_bf16(x)


def _parameters(product, net):
    count = product.fractal_gb300_costnet_parameter_count()
    assert count == oracle.PARAMS
    values = (ctypes.c_float * count)()
    assert product.fractal_gb300_costnet_parameters(net, values, count, 0) == 0, product.fractal_last_error()
    return np.frombuffer(values, dtype=np.float32).astype(np.float64)


def _train(product, net, x_dev, t_dev, batch, lr, update):
    count = product.fractal_gb300_costnet_parameter_count()
    grads = (ctypes.c_float * count)()
    loss = ctypes.c_float(0.0)
    status = product.fractal_gb300_costnet_train_step(net, x_dev.data_ptr(), t_dev.data_ptr(), batch, lr,
                                                      int(update), ctypes.byref(loss), grads, None)
    assert status == 0, product.fractal_last_error()
    return float(loss.value), np.frombuffer(grads, dtype=np.float32).astype(np.float64)


def test_costnet_forward_and_gradients_match_oracle(product):
    rng = np.random.default_rng(11)
    batch = 256
    net = product.fractal_gb300_costnet_create(5)
    assert net, product.fractal_last_error()
    try:
        params = _parameters(product, net)
        x = _features(rng, batch)
        t = rng.standard_normal(batch).astype(np.float32)
        x_dev = _bf16(x)
        t_dev = torch.from_numpy(t).cuda()
        y_dev = torch.empty(batch, dtype=torch.float32, device="cuda")
        assert product.fractal_gb300_costnet_predict(net, x_dev.data_ptr(), batch, y_dev.data_ptr(), None) == 0
        y_cpu, _ = oracle.forward(params, x)
        np.testing.assert_allclose(y_dev.cpu().numpy(), y_cpu, rtol=2e-2, atol=2e-3)
        loss, grads = _train(product, net, x_dev, t_dev, batch, 0.0, False)
        loss_cpu, grads_cpu = oracle.loss_and_gradient(params, x, t)
        assert abs(loss - loss_cpu) <= 1e-3 * loss_cpu + 1e-6
        offsets = np.cumsum([0, 256 * 320, 256, 256 * 256, 256, 256, 1])
        for block, name in enumerate(["W1", "b1", "W2", "b2", "w3", "b3"]):
            g = grads[offsets[block]:offsets[block + 1]]
            c = grads_cpu[offsets[block]:offsets[block + 1]]
            error = np.linalg.norm(g - c) / max(np.linalg.norm(c), 1e-12)
            assert error <= 2e-2, (name, error)
        # Training leaves the gradient check untouched: no update was made.
        np.testing.assert_array_equal(_parameters(product, net), params)
    finally:
        product.fractal_gb300_costnet_destroy(net)


def test_costnet_adam_step_and_training(product):
    rng = np.random.default_rng(12)
    batch = 512
    net = product.fractal_gb300_costnet_create(9)
    assert net, product.fractal_last_error()
    try:
        x = _features(rng, batch)
        # A smooth target of the probe features (mean log count) and the zoom.
        t = (x[:, :256].mean(axis=1) * 4.0 + x[:, 256] - 2.0).astype(np.float32)
        x_dev = _bf16(x)
        t_dev = torch.from_numpy(t).cuda()
        params = _parameters(product, net)
        loss0, grads = _train(product, net, x_dev, t_dev, batch, 1e-3, True)
        expect, _, _ = oracle.adam_step(params, grads, np.zeros_like(params), np.zeros_like(params), 1, 1e-3)
        np.testing.assert_allclose(_parameters(product, net), expect, rtol=1e-5, atol=1e-7)
        loss = loss0
        for _ in range(300):
            loss, _ = _train(product, net, x_dev, t_dev, batch, 1e-3, True)
        assert loss < 0.05 * loss0, (loss0, loss)
    finally:
        product.fractal_gb300_costnet_destroy(net)


@pytest.mark.parametrize("key,log_zoom,cap", [("field_e100", 100.0, 1_000_000), ("deep_nucleus_p80", 32.8, 100_000)],
                         ids=["uniform_e100", "minibrot_e32"])
def test_learned_order_on_8k_field_keeps_pixels_and_reports_gain(package, product, key, log_zoom, cap):
    """7680x4320 fields: the uniform view at 1e100 (cap 1e6) and a view of the
    period-80 minibrot at 1e32.8 (cap 1e5; tile costs vary, about half of the
    pixels are strict glitches near the minibrot).  Pixel-chunk queue, static
    tile order and the trained network's heaviest-first order render
    identical pixels; the makespan and tail of both tile orders are printed
    and the learned order may not be slower than the static one beyond
    noise."""
    import json

    native = package.native
    atlas = package.atlas
    net = package.costnet.load_default(product)
    with open(os.path.join(ROOT, "tests", "golden", "centres.json"), encoding="ascii") as handle:
        centre = json.load(handle)[key]
    width, height = 7680, 4320
    bits = atlas.precision_bits(centre["re"], centre["im"], log_zoom)
    handle = native.create_reference(product, centre["re"], centre["im"], atlas.zoom_text(log_zoom), cap, bits, 32)
    field = torch.empty(width * height, dtype=torch.float32, device="cuda")
    counts = torch.empty(width * height, dtype=torch.int32, device="cuda")
    frames = (native.Keyframe * 1)()
    zoom = atlas.zoom_text(log_zoom)
    frames[0].field = field.data_ptr()
    frames[0].counts = counts.data_ptr()
    frames[0].zoom_text = zoom
    frames[0].reference = handle
    frames[0].max_iter = cap
    options = native.RenderOptions()

    def render(flags):
        status = product.fractal_gb300_render_keyframes_device(frames, 1, width, height, None, None, 3, 256,
                                                               ctypes.byref(options), 1, flags, None)
        assert status == 0, native.last_error(product)
        torch.cuda.synchronize()
        timing = (ctypes.c_double * 2)()
        if flags & native.BATCH_TILES:
            assert product.fractal_gb300_last_tiles(None, None, None, 0, timing) == 0, native.last_error(product)
        return field.cpu().numpy().view(np.uint32).copy(), counts.cpu().numpy().copy(), (timing[0], timing[1])

    try:
        net.attach()
        want_field, want_counts, _ = render(0)
        results = {}
        for name, flags in (("static", native.BATCH_TILES), ("learned", native.BATCH_TILES | native.BATCH_LEARNED)):
            runs = []
            for _ in range(3):
                got_field, got_counts, timing = render(flags)
                np.testing.assert_array_equal(got_counts, want_counts)
                np.testing.assert_array_equal(got_field, want_field)
                runs.append(timing)
            results[name] = sorted(runs)[1]
        print(f"8K {key} 1e{log_zoom} cap {cap}: static makespan {results['static'][0]:.2f} ms tail {results['static'][1]:.2f} ms; "
              f"learned makespan {results['learned'][0]:.2f} ms tail {results['learned'][1]:.2f} ms")
        assert results["learned"][0] <= results["static"][0] * 1.05 + 0.5
    finally:
        product.fractal_gb300_set_cost_network(None)
        net.close()
        product.fractal_destroy_reference(handle)
