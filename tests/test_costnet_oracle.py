"""CPU: the tile-cost network oracle's gradient against central differences.

oracle/costnet.py is the reference the GPU gradients are checked against, so
its own derivative is pinned here in float64 (no BF16 rounding), at random
parameter coordinates of every block.
"""

from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import costnet as oracle  # noqa: E402


def test_bf16_rounding_is_nearest_even():
    values = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e38, 1e-40, 0.0], dtype=np.float32)
    rounded = oracle.round_bf16(values)
    assert rounded[0] == 1.0
    assert rounded[1] == 1.0                 # halfway 1 + 2^-8: to even (1.0)
    assert rounded[2] == np.float32(1.0078125)  # above halfway: up
    assert rounded[3] == -2.5
    assert np.isfinite(rounded[4])
    assert rounded[6] == 0.0


def test_oracle_gradient_matches_central_differences():
    rng = np.random.default_rng(7)
    batch = 16
    x = rng.standard_normal((batch, oracle.FEATURES)) * 0.5
    x[:, 258:] = 0.0
    t = rng.standard_normal(batch)
    params = rng.standard_normal(oracle.PARAMS) * 0.05
    loss, grad = oracle.loss_and_gradient(params, x, t, bf16=False)
    assert np.isfinite(loss)
    offsets = np.cumsum([0, 256 * 320, 256, 256 * 256, 256, 256, 1])
    eps = 1e-6
    for block in range(6):
        for index in rng.integers(offsets[block], offsets[block + 1], size=4):
            if block == 0 and (index % 320) >= 258:
                continue
            up = params.copy()
            up[index] += eps
            down = params.copy()
            down[index] -= eps
            numeric = (oracle.loss_and_gradient(up, x, t, bf16=False)[0]
                       - oracle.loss_and_gradient(down, x, t, bf16=False)[0]) / (2 * eps)
            assert abs(numeric - grad[index]) <= 1e-6 + 1e-4 * abs(numeric), (block, index, numeric, grad[index])
