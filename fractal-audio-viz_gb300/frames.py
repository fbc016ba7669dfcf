"""Video-frame handoff to an encoder pipe (the reference's FFmpeg writer,
visualizer.py:3203-3260): each device RGB8 frame is packed on the GPU
(fractal_gb300_pack_frame_device) into the pipe's layout and copied into one
of two pinned host buffers on a side stream, so frame t's copy and write
overlap frame t+1's rendering.
"""

from __future__ import annotations

import ctypes

from . import native

FORMATS = {"rgb24": 0, "rgb0": 1, "rgba": 2, "yuv420p": 3, "nv12": 4}


class FrameWriter:
    """Writes packed frames to `sink` (a binary file object: FFmpeg's stdin).

    ``push(rgb_ptr, stream)`` enqueues a frame held in device memory behind
    the work already on `stream`; ``close()`` drains and flushes.
    """

    def __init__(self, library, sink, width: int, height: int, pixel_format: str = "rgb24"):
        import torch

        if pixel_format not in FORMATS:
            raise ValueError(f"unknown pixel format {pixel_format!r}")
        self.library = library
        self.sink = sink
        self.width = width
        self.height = height
        self.format = FORMATS[pixel_format]
        size = library.fractal_gb300_packed_frame_bytes(width, height, self.format)
        if size <= 0:
            raise native.NativeError("invalid frame size or format")
        self.frame_bytes = int(size)
        self.device = [torch.empty(self.frame_bytes, dtype=torch.uint8, device="cuda") for _ in range(2)]
        self.host = [torch.empty(self.frame_bytes, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        self.copy_stream = torch.cuda.Stream()
        self.done = [None, None]
        self.slot = 0
        self.frames = 0

    def _drain(self, slot: int) -> None:
        event = self.done[slot]
        if event is not None:
            event.synchronize()
            self.sink.write(memoryview(self.host[slot].numpy()))
            self.done[slot] = None

    def push(self, rgb_ptr: int, stream) -> None:
        import torch

        slot = self.slot
        self._drain(slot)
        status = self.library.fractal_gb300_pack_frame_device(
            ctypes.c_void_p(rgb_ptr), self.width, self.height, self.format,
            ctypes.c_void_p(self.device[slot].data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        if status != 0:
            raise native.NativeError(native.last_error(self.library))
        packed = torch.cuda.Event()
        packed.record(stream)
        self.copy_stream.wait_event(packed)
        with torch.cuda.stream(self.copy_stream):
            self.host[slot].copy_(self.device[slot], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.copy_stream)
        self.done[slot] = done
        self.slot = 1 - slot
        self.frames += 1

    def close(self) -> None:
        self._drain(self.slot)
        self._drain(1 - self.slot)
        if hasattr(self.sink, "flush"):
            self.sink.flush()
