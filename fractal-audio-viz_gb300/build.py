"""Build the GB300 renderer library in-tree: ``_build/libfractal_gb300.so``.

Every translation unit is compiled for sm_103a only, in parallel, without
cmake.  The plain-form kernels and all host table builders are compiled
without floating-point contraction (``--fmad=false`` / ``-ffp-contract=off``)
so that their double arithmetic rounds operation by operation like the
reference release build; the floatexp and colour kernels use FMA freely.

Usage:  python fractal-audio-viz_gb300/build.py [--force] [--jobs N]
"""

from __future__ import annotations

import argparse
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIBRARY = os.path.join(BUILD, "libfractal_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Translation units compiled with contraction allowed (FP32 floatexp, colour).
FMA_UNITS = {"render_fe.cu", "colour_kfp.cu", "mlp.cu"}


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _sources():
    names = sorted(os.listdir(CSRC))
    return [n for n in names if n.endswith((".cu", ".cpp"))]


def _headers_mtime() -> float:
    newest = 0.0
    for directory in (CSRC, INCLUDE):
        for name in os.listdir(directory):
            if name.endswith((".h", ".cuh")):
                newest = max(newest, os.path.getmtime(os.path.join(directory, name)))
    return newest


def _compile(name: str, force: bool, header_time: float, cuda_home: str) -> str:
    source = os.path.join(CSRC, name)
    obj = os.path.join(BUILD, name + ".o")
    if (not force and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(source), header_time)):
        return obj
    includes = ["-I" + CSRC, "-I" + INCLUDE]
    if name.endswith(".cu"):
        fmad = "true" if name in FMA_UNITS else "false"
        command = ["nvcc", *ARCH, "-O3", "-lineinfo", "-std=c++17", f"--fmad={fmad}",
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills",
                   *includes, "-c", source, "-o", obj]
    else:
        command = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
                   "-I" + os.path.join(cuda_home, "include"), *includes, "-c", source, "-o", obj]
    result = subprocess.run(command, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"compile failed: {name}\n{' '.join(command)}\n{result.stdout}{result.stderr}")
    if result.stderr.strip():
        sys.stderr.write(result.stderr)
    return obj


def build(force: bool = False, jobs: int = 0) -> str:
    """Compile every source and link the shared library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    cuda_home = _cuda_home()
    header_time = _headers_mtime()
    sources = _sources()
    jobs = jobs or min(len(sources), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as pool:
        objects = list(pool.map(lambda n: _compile(n, force, header_time, cuda_home), sources))
    newest = max(os.path.getmtime(o) for o in objects)
    if force or not os.path.exists(LIBRARY) or os.path.getmtime(LIBRARY) < newest:
        command = ["nvcc", *ARCH, "-shared", "-cudart=static", "-o", LIBRARY, *objects, "-ldl", "-lpthread"]
        result = subprocess.run(command, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"link failed\n{' '.join(command)}\n{result.stdout}{result.stderr}")
    return LIBRARY


def main() -> int:
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--force", action="store_true")
    parser.add_argument("--jobs", type=int, default=0)
    args = parser.parse_args()
    print(build(force=args.force, jobs=args.jobs))
    return 0


if __name__ == "__main__":
    sys.exit(main())
