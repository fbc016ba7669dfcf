"""CPU oracle of the tile-cost network (test infrastructure only).

Restates the forward pass, the mean-squared-error gradient and one Adam step
of fractal-audio-viz_gb300/csrc/costnet.cu in float64 numpy, rounding to
BF16 (round to nearest even) exactly where the GPU stores BF16: the weight
copies W1, W2, w3, the activations h1, h2 and the layer gradients dZ2, dZ1.
The network has no counterpart in the reference; this file exists so the
GPU gradients can be checked (tests/test_gpu_costnet.py) and is itself
checked against central differences in float64 (tests/test_costnet_oracle.py).
Nothing in the library imports it.
"""

from __future__ import annotations

import numpy as np

FEATURES = 320
HIDDEN = 256
PARAMS = HIDDEN * FEATURES + HIDDEN + HIDDEN * HIDDEN + HIDDEN + HIDDEN + 1


def to_bf16_bits(values) -> np.ndarray:
    """float32 -> BF16 bit patterns (uint16), round to nearest even."""
    bits = np.ascontiguousarray(values, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounded = (bits + 0x7FFF + ((bits >> 16) & 1)) >> 16
    nan = np.isnan(np.asarray(values, dtype=np.float32))
    out = rounded.astype(np.uint16)
    out[nan] = 0x7FC0
    return out


def from_bf16_bits(bits) -> np.ndarray:
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def round_bf16(values) -> np.ndarray:
    return from_bf16_bits(to_bf16_bits(values))


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    i = 0

    def take(n, shape):
        nonlocal i
        block = p[i:i + n].reshape(shape)
        i += n
        return block

    w1 = take(HIDDEN * FEATURES, (HIDDEN, FEATURES))
    b1 = take(HIDDEN, (HIDDEN,))
    w2 = take(HIDDEN * HIDDEN, (HIDDEN, HIDDEN))
    b2 = take(HIDDEN, (HIDDEN,))
    w3 = take(HIDDEN, (HIDDEN,))
    b3 = take(1, (1,))
    return w1, b1, w2, b2, w3, b3


def pack(w1, b1, w2, b2, w3, b3) -> np.ndarray:
    return np.concatenate([np.ravel(v) for v in (w1, b1, w2, b2, w3, b3)])


def _r(values, bf16: bool):
    if not bf16:
        return np.asarray(values, dtype=np.float64)
    return round_bf16(np.asarray(values, dtype=np.float32)).astype(np.float64)


def forward(params, x, *, bf16: bool = True):
    """Predictions and the intermediates backward() needs."""
    w1, b1, w2, b2, w3, b3 = unpack(params)
    w1q, w2q, w3q = _r(w1, bf16), _r(w2, bf16), _r(w3, bf16)
    x = np.asarray(x, dtype=np.float64)
    h1 = _r(np.maximum(x @ w1q.T + b1, 0.0), bf16)
    h2 = _r(np.maximum(h1 @ w2q.T + b2, 0.0), bf16)
    y = h2 @ w3q + b3[0]
    return y, (x, h1, h2, w2q, w3q)


def loss_and_gradient(params, x, target, *, bf16: bool = True):
    """Mean squared error and its gradient in parameter order."""
    y, (x, h1, h2, w2q, w3q) = forward(params, x, bf16=bf16)
    t = np.asarray(target, dtype=np.float64)
    batch = y.shape[0]
    diff = y - t
    loss = float(np.mean(diff * diff))
    dy = 2.0 * diff / batch
    gw3 = h2.T @ dy
    gb3 = np.array([dy.sum()])
    dz2 = _r(np.where(h2 > 0.0, dy[:, None] * w3q[None, :], 0.0), bf16)
    gw2 = dz2.T @ h1
    gb2 = dz2.sum(axis=0)
    dz1 = _r(np.where(h1 > 0.0, dz2 @ w2q, 0.0), bf16)
    gw1 = dz1.T @ x
    gb1 = dz1.sum(axis=0)
    return loss, pack(gw1, gb1, gw2, gb2, gw3, gb3)


def adam_step(params, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (returns new params, m, v)."""
    m = beta1 * m + (1.0 - beta1) * grad
    v = beta2 * v + (1.0 - beta2) * grad * grad
    c1 = 1.0 - beta1 ** step
    c2 = 1.0 - beta2 ** step
    return params - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v
