"""GPU: video-frame packing and the pinned double-buffered frame writer.

fractal_gb300_pack_frame_device equals the numpy restatement
(oracle/pack.py) byte for byte for every format on odd and even frame sizes;
FrameWriter delivers exactly the concatenated packed frames, in order.
"""

from __future__ import annotations

import ctypes
import importlib.util
import io
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle():
    spec = importlib.util.spec_from_file_location("oracle_pack", os.path.join(ROOT, "oracle", "pack.py"))
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


@pytest.mark.parametrize("size", [(3840, 2160), (1924, 1082), (4, 2), (1922, 1080), (1921, 1081), (7, 5)])
@pytest.mark.parametrize("fmt", ["rgb24", "rgb0", "rgba", "yuv420p", "nv12"])
def test_pack_matches_oracle(product, size, fmt):
    import torch

    oracle = _oracle()
    width, height = size
    rgb = np.random.default_rng(width + height).integers(0, 256, size=width * height * 3, dtype=np.uint8)
    d_rgb = torch.from_numpy(rgb).cuda()
    code = oracle.FORMATS[fmt]
    n = product.fractal_gb300_packed_frame_bytes(width, height, code)
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    status = product.fractal_gb300_pack_frame_device(ctypes.c_void_p(d_rgb.data_ptr()), width, height, code,
                                                     ctypes.c_void_p(out.data_ptr()), None)
    assert status == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), oracle.pack(rgb, width, height, fmt))


def test_frame_writer_order(product, package):
    import torch

    oracle = _oracle()
    width, height = 64, 36
    frames = [np.random.default_rng(k).integers(0, 256, size=width * height * 3, dtype=np.uint8) for k in range(5)]
    sink = io.BytesIO()
    stream = torch.cuda.Stream()
    writer = package.frames.FrameWriter(product, sink, width, height, "nv12")
    device = [torch.from_numpy(f).cuda() for f in frames]
    torch.cuda.synchronize()
    for d in device:
        writer.push(d.data_ptr(), stream)
    writer.close()
    want = b"".join(oracle.pack(f, width, height, "nv12").tobytes() for f in frames)
    assert sink.getvalue() == want
