"""ORACLE - test infrastructure only.

numpy restatement of the video-frame packing of the GB300 library
(rgb24 / rgb0 / rgba / yuv420p / nv12).  The reference hands rgb24 or rgb0 to
FFmpeg (visualizer.py:3203-3260, 12916-12942); those byte layouts are pinned
by that definition.  The YUV layouts have no counterpart in the reference
(FFmpeg's own converter is outside it): parity unpinned, this restates the
library's stated BT.709 integer form so the device kernel is checked against
it.
"""

from __future__ import annotations

import numpy as np

FORMATS = {"rgb24": 0, "rgb0": 1, "rgba": 2, "yuv420p": 3, "nv12": 4}


def _yuv(r, g, b):
    y = 16 + ((47 * r + 157 * g + 16 * b + 128) >> 8)
    u = 128 + ((-26 * r - 86 * g + 112 * b + 128) >> 8)
    v = 128 + ((112 * r - 102 * g - 10 * b + 128) >> 8)
    return y, u, v


def pack(rgb: np.ndarray, width: int, height: int, fmt: str) -> np.ndarray:
    image = np.asarray(rgb, dtype=np.uint8).reshape(height, width, 3)
    if fmt == "rgb24":
        return image.reshape(-1).copy()
    if fmt in ("rgb0", "rgba"):
        out = np.empty((height, width, 4), dtype=np.uint8)
        out[..., :3] = image
        out[..., 3] = 0 if fmt == "rgb0" else 255
        return out.reshape(-1)
    channels = image.astype(np.int64)
    y_plane, _, _ = _yuv(channels[..., 0], channels[..., 1], channels[..., 2])
    ch, cw = (height + 1) // 2, (width + 1) // 2
    sums = np.zeros((ch, cw, 3), dtype=np.int64)
    counts = np.zeros((ch, cw), dtype=np.int64)
    for dy in range(2):
        for dx in range(2):
            part = channels[dy::2, dx::2]
            sums[: part.shape[0], : part.shape[1]] += part
            counts[: part.shape[0], : part.shape[1]] += 1
    mean = (sums + (counts // 2)[..., None]) // counts[..., None]
    _, u, v = _yuv(mean[..., 0], mean[..., 1], mean[..., 2])
    parts = [y_plane.astype(np.uint8).reshape(-1)]
    if fmt == "yuv420p":
        parts += [u.astype(np.uint8).reshape(-1), v.astype(np.uint8).reshape(-1)]
    else:
        parts.append(np.stack([u, v], axis=-1).astype(np.uint8).reshape(-1))
    return np.concatenate(parts)
