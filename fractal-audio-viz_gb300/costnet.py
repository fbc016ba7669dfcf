"""Tile-cost network: training data, training and loading (host side).

The network (csrc/costnet.cu, csrc/mlp.cu) predicts the render cost of a
64x64 tile of a floatexp field from a 16x16 coarse probe of its iteration
counts plus the field's log zoom and cap; the persistent floatexp queue then
claims the heaviest tiles first (FRACTAL_GB300_BATCH_LEARNED).  It orders
work only: every pixel is the same as with the static order.

Training data are fields the renderer itself produces: seeded Misiurewicz
centres (costnet_centres.json, made by tests/golden/make_costnet_centres.py), each
rendered as one 1920x1080 atlas keyframe at a seeded level of the FHD ladder
(zoom 8^level, cap 2000 + 3000 per decade) through the tile queue in static
order with the probe on.  Labels are the measured per-tile costs (SM cycles)
as normalised logarithms; the network is trained on the GPU by its own
forward/backward kernels (Adam, mean squared error).

    python -m fractal_audio_viz_gb300.costnet   (or: python costnet.py)

trains on the default 200 fields and writes costnet_weights.npz beside this
file; load_default() attaches those weights to a library.
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import time
from dataclasses import dataclass

import numpy as np

from . import atlas, native

HERE = os.path.dirname(os.path.abspath(__file__))
CENTRES = os.path.join(HERE, "costnet_centres.json")
WEIGHTS = os.path.join(HERE, "costnet_weights.npz")
FEATURES = 320
TILE = 64


def _bf16_bits(values: np.ndarray) -> np.ndarray:
    bits = np.ascontiguousarray(values, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)


class CostNet:
    """A network on the GPU (fractal_gb300_costnet_*) with its target scale."""

    def __init__(self, library, seed: int = 1):
        self.library = library
        self.handle = library.fractal_gb300_costnet_create(seed)
        if not self.handle:
            raise native.NativeError(native.last_error(library))
        self.mean = 0.0
        self.std = 1.0

    def close(self) -> None:
        if self.handle:
            self.library.fractal_gb300_costnet_destroy(self.handle)
            self.handle = None

    def parameters(self) -> np.ndarray:
        count = self.library.fractal_gb300_costnet_parameter_count()
        values = (ctypes.c_float * count)()
        if self.library.fractal_gb300_costnet_parameters(self.handle, values, count, 0) != 0:
            raise native.NativeError(native.last_error(self.library))
        return np.frombuffer(values, dtype=np.float32).copy()

    def set_parameters(self, values: np.ndarray) -> None:
        values = np.ascontiguousarray(values, dtype=np.float32)
        buffer = values.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        if self.library.fractal_gb300_costnet_parameters(self.handle, buffer, values.size, 1) != 0:
            raise native.NativeError(native.last_error(self.library))

    def save(self, path: str) -> None:
        np.savez_compressed(path, parameters=self.parameters(), mean=self.mean, std=self.std)

    def load(self, path: str) -> None:
        with np.load(path) as data:
            self.set_parameters(data["parameters"])
            self.mean = float(data["mean"])
            self.std = float(data["std"])

    def attach(self) -> None:
        """Use this network for FRACTAL_GB300_BATCH_LEARNED on this thread."""
        if self.library.fractal_gb300_set_cost_network(self.handle) != 0:
            raise native.NativeError(native.last_error(self.library))

    def train(self, features: np.ndarray, targets: np.ndarray, *, epochs: int = 20, batch: int = 1024,
              learning_rate: float = 1e-3, seed: int = 0, log=None) -> list[float]:
        """Adam on mean squared error over (BF16 feature rows, normalised
        targets) held on the device; returns the per-epoch mean loss."""
        import torch

        rows = features.shape[0]
        usable = rows - rows % batch
        if usable <= 0:
            raise ValueError("fewer training rows than one batch")
        x = torch.from_numpy(features.astype(np.int16).view(np.int16)).cuda()
        t = torch.from_numpy(targets.astype(np.float32)).cuda()
        rng = np.random.default_rng(seed)
        history = []
        loss = ctypes.c_float(0.0)
        for epoch in range(epochs):
            order = torch.from_numpy(rng.permutation(rows)[:usable]).cuda()
            xs = x[order].contiguous()
            ts = t[order].contiguous()
            total = 0.0
            for start in range(0, usable, batch):
                status = self.library.fractal_gb300_costnet_train_step(
                    self.handle, xs[start:start + batch].data_ptr(), ts[start:start + batch].data_ptr(), batch,
                    learning_rate, 1, ctypes.byref(loss), None, None)
                if status != 0:
                    raise native.NativeError(native.last_error(self.library))
                total += loss.value
            history.append(total / (usable // batch))
            if log:
                log(f"epoch {epoch}: loss {history[-1]:.4f}")
        return history

    def predict(self, features: np.ndarray) -> np.ndarray:
        import torch

        rows = features.shape[0]
        padded = (rows + 127) // 128 * 128
        x = torch.zeros((padded, FEATURES), dtype=torch.int16, device="cuda")
        x[:rows] = torch.from_numpy(features.astype(np.int16).view(np.int16)).cuda()
        out = torch.empty(padded, dtype=torch.float32, device="cuda")
        if self.library.fractal_gb300_costnet_predict(self.handle, x.data_ptr(), padded, out.data_ptr(), None) != 0:
            raise native.NativeError(native.last_error(self.library))
        return out[:rows].cpu().numpy()


def load_default(library, path: str = WEIGHTS) -> CostNet:
    net = CostNet(library)
    net.load(path)
    return net


@dataclass
class TrainingField:
    centre: dict
    level: int
    log10_zoom: float
    cap: int


def training_fields(count: int = 200, seed: int = 2024) -> list[TrainingField]:
    """Seeded (centre, atlas level) pairs: level ~ U{14..54} of the FHD
    ladder (zoom 8^level; the deep, floatexp part of the atlas)."""
    with open(CENTRES, encoding="ascii") as handle:
        centres = json.load(handle)["centres"]
    rng = np.random.default_rng(seed)
    step = math.log10(8.0)
    fields = []
    for i in range(count):
        level = int(rng.integers(14, 55))
        log_zoom = level * step
        cap = min(200_000, max(64, int(2000 + 3000 * min(50.0, (level + 1) * step))))
        fields.append(TrainingField(centres[i % len(centres)], level, log_zoom, cap))
    return fields


def render_tiles(library, fields: list[TrainingField], width: int = 1920, height: int = 1080, *,
                 flags: int = native.BATCH_TILES | native.BATCH_PROBE, group: int = 8, stream=None,
                 measure: bool = True):
    """Render the fields through the tile queue; returns (features [N x 320]
    BF16 bits, per-tile cost in SM cycles, [(makespan ms, tail ms)]).

    With `measure` the queue runs one block (one warp per SM sub-partition)
    per SM while the costs are recorded, so a tile's cycle count is its own
    work rather than its share of a crowded SM; the pixels are the same."""
    import torch

    if measure:
        shapes = (ctypes.c_int * 4)(64, 0, 256, 1)
        if library.fractal_gb300_set_queue_shapes(shapes, 4) != 0:
            raise native.NativeError(native.last_error(library))
    try:
        return _render_tiles(library, fields, width, height, flags, group, stream)
    finally:
        if measure:
            library.fractal_gb300_set_queue_shapes(None, 0)


def _render_tiles(library, fields, width, height, flags, group, stream):
    import torch

    features, costs, timings = [], [], []
    tiles_per_field = ((width + TILE - 1) // TILE) * ((height + TILE - 1) // TILE)
    for start in range(0, len(fields), group):
        chunk = fields[start:start + group]
        handles = []
        try:
            for f in chunk:
                bits = atlas.precision_bits(f.centre["re"], f.centre["im"], f.log10_zoom)
                handles.append(native.create_reference(library, f.centre["re"], f.centre["im"],
                                                       atlas.zoom_text(f.log10_zoom), f.cap, bits, 32))
            field = torch.empty((len(chunk), width * height), dtype=torch.float32, device="cuda")
            counts = torch.empty((len(chunk), width * height), dtype=torch.int32, device="cuda")
            frames = (native.Keyframe * len(chunk))()
            zooms = [atlas.zoom_text(f.log10_zoom) for f in chunk]
            for i, f in enumerate(chunk):
                frames[i].field = field[i].data_ptr()
                frames[i].counts = counts[i].data_ptr()
                frames[i].zoom_text = zooms[i]
                frames[i].reference = handles[i]
                frames[i].max_iter = f.cap
            options = native.RenderOptions()
            status = library.fractal_gb300_render_keyframes_device(
                frames, len(chunk), width, height, None, None, 3, 256, ctypes.byref(options), 1, flags,
                ctypes.c_void_p(stream))
            if status != 0:
                raise native.NativeError(native.last_error(library))
            n = tiles_per_field * len(chunk)
            tiles = ctypes.c_int(0)
            cost = np.zeros(n, dtype=np.float32)
            feats = np.zeros((n, FEATURES), dtype=np.uint16)
            timing = (ctypes.c_double * 2)()
            if library.fractal_gb300_last_tiles(ctypes.byref(tiles), cost.ctypes.data, feats.ctypes.data, n,
                                                timing) != 0:
                raise native.NativeError(native.last_error(library))
            features.append(feats[:tiles.value])
            costs.append(cost[:tiles.value])
            timings.append((timing[0], timing[1]))
        finally:
            for h in handles:
                library.fractal_destroy_reference(h)
    return np.concatenate(features), np.concatenate(costs), timings


def normalise(costs: np.ndarray):
    logs = np.log(np.maximum(costs, 1.0))
    mean = float(logs.mean())
    std = float(logs.std()) or 1.0
    return (logs - mean) / std, mean, std


def main() -> None:
    import argparse

    from . import load_library

    parser = argparse.ArgumentParser(description="train the tile-cost network on rendered fields")
    parser.add_argument("--fields", type=int, default=200)
    parser.add_argument("--epochs", type=int, default=30)
    parser.add_argument("--out", default=WEIGHTS)
    args = parser.parse_args()
    library = load_library()
    t0 = time.perf_counter()
    fields = training_fields(args.fields)
    features, costs, _ = render_tiles(library, fields)
    print(f"collected {len(costs)} tiles from {len(fields)} fields in {time.perf_counter() - t0:.1f} s", flush=True)
    targets, mean, std = normalise(costs)
    net = CostNet(library, seed=1)
    net.mean, net.std = mean, std
    history = net.train(features, targets, epochs=args.epochs, log=print)
    net.save(args.out)
    print(json.dumps({"tiles": int(len(costs)), "final_loss": history[-1], "mean": mean, "std": std}))
    net.close()


if __name__ == "__main__":
    main()
