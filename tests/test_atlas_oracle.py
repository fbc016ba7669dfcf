"""Pin the atlas compositor of the oracle port to the reference.

Every case of ``golden/atlas_cases.py`` through the port's
fractal_atlas_field[_ex] / fractal_atlas_colourise[_interior|_accents] /
fractal_colourise_accents must reproduce the reference release build's
stored output bit for bit (``golden/fixtures/atlas.npz``).  The port has no
KFP colour pass; its scalar surfaces (oracle_atlas_kfp_surface,
oracle_crop_kfp_surface) are pinned instead: the reference's own KFP pass over
a surface must give exactly the reference's fractal_atlas_colourise_kfp_raw /
fractal_crop_colourise_kfp frame.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from .golden import atlas_cases


@pytest.fixture(scope="module")
def atlas_fixture():
    with np.load(atlas_cases.ATLAS_FIXTURE) as data:
        return {key: data[key] for key in data.files}


PORT_CASES = [c for c in atlas_cases.CASES if c["kind"] not in ("kfp_raw", "crop_kfp")]
KFP_CASES = [c for c in atlas_cases.CASES if c["kind"] in ("kfp_raw", "crop_kfp")]


def oracle_surface(port, case):
    """The port's scalar surface of a raw KFP atlas or KFP crop case (the
    float32 frame the KFP pass colours)."""
    f32 = ctypes.POINTER(ctypes.c_float)
    if case.get("kind") == "crop_kfp":
        port.oracle_crop_kfp_surface.restype = ctypes.c_int
        port.oracle_crop_kfp_surface.argtypes = [f32, ctypes.c_int, ctypes.c_int, f32, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_double, ctypes.c_int, ctypes.c_double]
        source, shape, _ = atlas_cases.source(case["parent"])
        width, height = case["output"]
        out = np.empty(width * height, dtype=np.float32)
        status = port.oracle_crop_kfp_surface(source.ctypes.data_as(f32), shape[0], shape[1], out.ctypes.data_as(f32),
                                              width, height, case["parent_zoom"], case["max_iter"],
                                              case["field_bias"])
        assert status == 0, port.fractal_last_error()
        return out
    port.oracle_atlas_kfp_surface.restype = ctypes.c_int
    port.oracle_atlas_kfp_surface.argtypes = [f32, ctypes.c_int, ctypes.c_int, ctypes.c_int, f32, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, f32, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                              ctypes.c_double]
    parent, parent_shape, parent_cap, child, child_shape, child_cap = atlas_cases.inputs(case)
    width, height = case["output"]
    out = np.empty(width * height, dtype=np.float32)
    cw, ch = child_shape if child is not None else (0, 0)
    status = port.oracle_atlas_kfp_surface(
        parent.ctypes.data_as(f32), parent_shape[0], parent_shape[1], parent_cap,
        child.ctypes.data_as(f32) if child is not None else None, cw, ch, child_cap, out.ctypes.data_as(f32),
        width, height, case["parent_zoom"], case["fraction"], case["child_zoom"], case["max_iter"],
        case["field_bias"])
    assert status == 0, port.fractal_last_error()
    return out


@pytest.mark.parametrize("case", KFP_CASES, ids=lambda c: c["name"])
def test_port_kfp_surface_pins_reference(oracle_port, reference_library, package, atlas_fixture, case):
    surface = oracle_surface(oracle_port, case)
    options, lut = atlas_cases.kfp_inputs(case)
    width, height = case["output"]
    rgb = np.empty(width * height * 3, dtype=np.uint8)
    status = reference_library.fractal_colourise_kfp(
        surface.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), rgb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
        width, height, case["max_iter"], 0.0, 0.0, 0.0, 0.5, ctypes.byref(options),
        lut.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), lut.shape[0], 0)
    assert status == 0, package.native.last_error(reference_library)
    np.testing.assert_array_equal(rgb, atlas_fixture[case["name"]])


@pytest.mark.parametrize("case", PORT_CASES, ids=lambda c: c["name"])
def test_port_atlas_matches_reference_fixture(oracle_port, atlas_fixture, case):
    out = atlas_cases.run(oracle_port, case)
    expected = atlas_fixture[case["name"]]
    assert out.dtype == expected.dtype and out.shape == expected.shape
    np.testing.assert_array_equal(out.view(np.uint8), expected.view(np.uint8))


def test_port_atlas_rejects_what_the_reference_rejects(oracle_port, reference_library, package):
    native = package.native
    parent = np.zeros(16 * 9, dtype=np.float32)
    bad = [
        dict(parent_zoom=0.0),
        dict(child_fraction=1.5),
        dict(output_bias=1e9),
        dict(parent_bias=-1.0),
        dict(feather=-1),
    ]
    for change in bad:
        kwargs = dict(parent_zoom=1.0, child_fraction=0.5, child_zoom=1.0, parent_bias=0.0, child_bias=0.0,
                      output_bias=0.0, feather=48)
        kwargs.update(change)
        for library in (oracle_port, reference_library):
            with pytest.raises(native.NativeError):
                native.atlas_field(library, parent, (16, 9), 100, parent, (16, 9), 100, (16, 9),
                                   kwargs["parent_zoom"],
                                   kwargs["child_fraction"], 100, child_zoom=kwargs["child_zoom"],
                                   parent_bias=kwargs["parent_bias"], child_bias=kwargs["child_bias"],
                                   output_bias=kwargs["output_bias"], feather=kwargs["feather"])
