"""GB300 deep-zoom field renderer: Python side of the renderer.h C ABI.

``build()`` compiles ``csrc/`` into ``_build/libfractal_gb300.so``;
``native`` holds the ctypes binding shared with the reference's ABI.  The
compute path is the CUDA library: importing this package never falls back to
a CPU renderer.
"""

from __future__ import annotations

import importlib.util
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))


def _load(name: str):
    full = f"{__name__}.{name}"
    if full in sys.modules:
        return sys.modules[full]
    spec = importlib.util.spec_from_file_location(full, os.path.join(_HERE, name + ".py"))
    module = importlib.util.module_from_spec(spec)
    sys.modules[full] = module
    spec.loader.exec_module(module)
    return module


native = _load("native")
atlas = _load("atlas")
kfp = _load("kfp")
costnet = _load("costnet")
frames = _load("frames")
fields = _load("fields")
song = _load("song")
_builder = _load("build")
LIBRARY_PATH = _builder.LIBRARY


def build(force: bool = False) -> str:
    """Compile the CUDA library for sm_103a (in-tree) and return its path."""
    return _builder.build(force=force)


def load_library(path: str | None = None):
    """Load the GB300 library (building it first when it is missing)."""
    if path is None:
        path = LIBRARY_PATH if os.path.exists(LIBRARY_PATH) else build()
    return native.load(path, gb300=True)
