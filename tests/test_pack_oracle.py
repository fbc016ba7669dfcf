"""The frame-packing oracle (oracle/pack.py): byte layouts and known values."""

from __future__ import annotations

import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _pack():
    spec = importlib.util.spec_from_file_location("oracle_pack", os.path.join(ROOT, "oracle", "pack.py"))
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


def test_rgb_layouts():
    pack = _pack()
    rgb = np.arange(2 * 3 * 3, dtype=np.uint8)
    assert np.array_equal(pack.pack(rgb, 3, 2, "rgb24"), rgb)
    rgb0 = pack.pack(rgb, 3, 2, "rgb0").reshape(-1, 4)
    assert np.array_equal(rgb0[:, :3].reshape(-1), rgb) and np.all(rgb0[:, 3] == 0)
    assert np.all(pack.pack(rgb, 3, 2, "rgba").reshape(-1, 4)[:, 3] == 255)


def test_yuv_known_values():
    pack = _pack()
    # Black, white, and the primaries land on BT.709 studio-swing values.
    for colour, expect in (((0, 0, 0), (16, 128, 128)), ((255, 255, 255), (235, 128, 128)),
                           ((255, 0, 0), (63, 102, 240)), ((0, 255, 0), (172, 42, 26)),
                           ((0, 0, 255), (32, 240, 118))):
        rgb = np.tile(np.array(colour, dtype=np.uint8), 4)
        out = pack.pack(rgb, 2, 2, "yuv420p")
        assert tuple(int(v) for v in (out[0], out[4], out[5])) == expect, colour


def test_yuv_sizes_odd_frames():
    pack = _pack()
    rgb = np.random.default_rng(0).integers(0, 256, size=5 * 3 * 3, dtype=np.uint8)
    assert pack.pack(rgb, 5, 3, "yuv420p").size == 15 + 2 * 3 * 2
    assert pack.pack(rgb, 5, 3, "nv12").size == 15 + 2 * 3 * 2
