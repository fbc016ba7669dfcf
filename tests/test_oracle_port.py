"""Pin the oracle port (oracle/oracle.cpp) to the reference.

The port is the CPU restatement used where the reference cannot be built.
Every Mandelbrot parity case must come out bit-identical to the golden
fixtures, which are the reference release build's own output.
"""

from __future__ import annotations

import math

import numpy as np
import pytest

from .conftest import golden_arrays
from .golden import cases as case_defs
from .golden.runner import run_case, summary

CASES = [c for c in case_defs.parity_cases() if c["formula"] == "mandelbrot"
         or c["kind"] == "direct"]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_port_matches_reference_fixture(oracle_port, golden_index, case):
    result = run_case(oracle_port, case)
    stored = golden_arrays(case["name"])
    if stored is None:
        assert summary(result) == golden_index[case["name"]]
        return
    np.testing.assert_array_equal(result["counts"], stored["counts"])
    np.testing.assert_array_equal(result["field"].view(np.uint32), stored["field"].view(np.uint32))
    if "orbit_iteration" in stored:
        for key in ("orbit_iteration", "phase", "de_x", "de_y", "test1", "test2"):
            np.testing.assert_array_equal(result[key], stored[key])


def test_port_aurora_matches_reference(oracle_port, reference_library, package):
    native = package.native
    stored = golden_arrays("e30_160x90")
    field = stored["field"]
    for controls in ((0.3, 0.4, 0.7, 0.5), (1.7, 0.9, 0.1, 0.05), (0.0, 0.0, 0.0, 0.95)):
        a = native.colourise(oracle_port, field, 160, 90, 50_000, *controls)
        b = native.colourise(reference_library, field, 160, 90, 50_000, *controls)
        np.testing.assert_array_equal(a, b)


def test_port_runs_at_reference_speed(oracle_port, reference_library, package):
    """The CPU baseline on the GPU host is the port (the reference sources are
    not there), so it must run at least at 0.9x the reference build's speed:
    both render the same deep levels of the FHD stack at 240x135 through the
    same ABI, interleaved, best of five each, on the same thread count."""
    import time

    from .golden import cases as case_defs

    native, atlas = package.native, package.atlas
    e50 = case_defs.centres()["fhd_stack_e50"]
    levels = [lv for lv in case_defs.fhd_stack_levels() if lv[0] in (30, 40, 54)]
    stacks = {name: atlas.KeyframeStack(lib, e50["re"], e50["im"], levels, step=math.log10(8.0))
              for name, lib in (("port", oracle_port), ("reference", reference_library))}
    best = {name: 0.0 for name in stacks}
    try:
        for _ in range(5):
            for name, stack in stacks.items():
                t0 = time.perf_counter()
                work = 0
                for keyframe in stack.keyframes:
                    field, planes = stack.render_host(keyframe, 240, 135, threads=2, planes=True)
                    work += int(native.iteration_counts(field, planes["orbit_iteration"], keyframe.max_iter)
                                .astype(np.uint64).sum())
                best[name] = max(best[name], work / (time.perf_counter() - t0))
    finally:
        for stack in stacks.values():
            stack.close()
    assert best["port"] >= 0.9 * best["reference"], best
