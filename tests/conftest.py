"""Shared fixtures: library loading, golden fixtures, markers.

``-m gpu`` tests need a CUDA device and call the GB300 library through its
C ABI.  Everything else runs on the CPU: oracle checks against the golden
fixtures, host-side logic, and the library's exports.
"""

from __future__ import annotations

import importlib.util
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PACKAGE_DIR = os.path.join(ROOT, "fractal-audio-viz_gb300")
FIXTURES = os.path.join(ROOT, "tests", "golden", "fixtures")
# The reference checkout (read-only; present only where the fixtures are made).
REFERENCE_SOURCES = os.environ.get("REFERENCE_DIR", "/root/reference")

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    """Import the package directory (its name is not a Python identifier)."""
    name = "fractal_audio_viz_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, os.path.join(PACKAGE_DIR, "__init__.py"), submodule_search_locations=[PACKAGE_DIR])
    module = importlib.util.module_from_spec(spec)
    sys.modules[name] = module
    spec.loader.exec_module(module)
    return module


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the C ABI")


@pytest.fixture(scope="session")
def package():
    return load_package()


@pytest.fixture(scope="session")
def product_path(package):
    return package.build()


@pytest.fixture(scope="session")
def product(package, product_path):
    return package.native.load(product_path, gb300=True)


@pytest.fixture(scope="session")
def golden_index():
    with open(os.path.join(FIXTURES, "index.json"), encoding="ascii") as handle:
        return json.load(handle)["cases"]


def golden_arrays(name: str):
    path = os.path.join(FIXTURES, name + ".npz")
    if not os.path.exists(path):
        return None
    with np.load(path) as data:
        return {key: data[key] for key in data.files}


@pytest.fixture(scope="session")
def reference_library(package):
    """The reference renderer compiled from its sources (oracle/_ref)."""
    path = os.path.join(ROOT, "oracle", "_ref", "mandelbrot.so")
    if not os.path.exists(path):
        if not os.path.isdir(REFERENCE_SOURCES):
            pytest.skip("reference sources are not present on this machine")
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True,
                       capture_output=True)
    return package.native.load(path)


@pytest.fixture(scope="session")
def oracle_port(package):
    """The CPU restatement of the path (oracle/oracle.cpp), built on demand."""
    path = os.path.join(ROOT, "oracle", "_ref", "liboracle.so")
    source = os.path.join(ROOT, "oracle", "oracle.cpp")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(source):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "port"], check=True,
                       capture_output=True)
    return package.native.load(path)
