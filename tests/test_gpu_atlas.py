"""GPU: the atlas compositor (compose.cu) against the reference and the oracle.

* every case of ``golden/atlas_cases.py`` reproduces the reference release
  build's stored frame bit for bit (scalar frames and aurora RGB8); raw KFP
  frames are within +-1 per channel with >= 99.9 % of bytes exact (the KFP
  colour pass computes its transcendentals in FP32), and their scalar
  surfaces equal the oracle port's bit for bit;
* full-size frames (3840x2160 from 1920x1080 parent and child fields with
  interior, NaN and +inf samples) equal the oracle port's frames bit for bit;
* invalid arguments fail with the reference's messages and leave the
  library usable.
"""

from __future__ import annotations

import numpy as np
import pytest

from .golden import atlas_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def atlas_fixture():
    with np.load(atlas_cases.ATLAS_FIXTURE) as data:
        return {key: data[key] for key in data.files}


@pytest.mark.parametrize("case", atlas_cases.CASES, ids=lambda c: c["name"])
def test_atlas_matches_reference_fixture(product, atlas_fixture, case):
    out = atlas_cases.run(product, case)
    expected = atlas_fixture[case["name"]]
    assert out.dtype == expected.dtype and out.shape == expected.shape
    if case["kind"] in ("kfp_raw", "crop_kfp"):
        diff = np.abs(out.astype(np.int16) - expected.astype(np.int16))
        assert diff.max() <= 1, f"max channel difference {diff.max()}"
        assert np.mean(diff == 0) >= 0.999, f"only {np.mean(diff == 0):.5f} of bytes exact"
        return
    mismatch = np.flatnonzero(out.view(np.uint8) != expected.view(np.uint8))
    assert mismatch.size == 0, f"{mismatch.size} bytes differ, first at {mismatch[:8]}"


def _device_surface(product, case, torch):
    parent, parent_shape, parent_cap, child, child_shape, child_cap = atlas_cases.inputs(case)
    d_parent = torch.from_numpy(parent).cuda()
    d_child = torch.from_numpy(child).cuda() if child is not None else None
    width, height = case["output"]
    out = torch.empty(width * height, dtype=torch.float32, device="cuda")
    cw, ch = child_shape if child is not None else (0, 0)
    status = product.fractal_gb300_atlas_kfp_surface_device(
        d_parent.data_ptr(), parent_shape[0], parent_shape[1], parent_cap,
        d_child.data_ptr() if d_child is not None else None, cw, ch, child_cap, out.data_ptr(), width, height,
        case["parent_zoom"], case["fraction"], case["child_zoom"], case["max_iter"], case["field_bias"], None)
    assert status == 0, product.fractal_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("case", [c for c in atlas_cases.CASES if c["kind"] == "kfp_raw"], ids=lambda c: c["name"])
def test_kfp_surface_matches_oracle(product, oracle_port, case):
    import torch

    from .test_atlas_oracle import oracle_surface

    got = _device_surface(product, case, torch)
    want = oracle_surface(oracle_port, case)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_kfp_surface_4k_matches_oracle(product, oracle_port):
    """3840x2160 raw KFP surfaces from 1920x1080 sources at several zoom
    phases, plain and centred encodings."""
    import torch

    from .test_atlas_oracle import oracle_surface

    parent = _structured_field(1920, 1080, 20000, 11)
    child = _structured_field(1920, 1080, 26000, 12)
    for zoom, fraction, bias in ((1.0, 0.25, 0.0), (2.0, 0.5, 0.0), (3.9, 0.975, 26000.0), (1.3, 1.0, 0.0)):
        case = dict(arrays=((parent, (1920, 1080), 20000), (child, (1920, 1080), 26000)), centred=bias > 0.0,
                    output=(3840, 2160), parent_zoom=zoom, fraction=fraction, child_zoom=1.0, max_iter=26000,
                    field_bias=bias)
        got = _device_surface(product, case, torch)
        want = oracle_surface(oracle_port, case)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def _structured_field(width, height, cap, seed):
    """A smooth banded field with interior discs, NaN streaks and +inf
    samples (seeded)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    base = 0.5 + 0.25 * np.sin(x / (17.0 + 5 * rng.uniform())) + 0.25 * np.cos(y / (23.0 + 5 * rng.uniform()))
    field = (base * 0.9 * cap).astype(np.float32)
    for _ in range(12):
        cx, cy, r = rng.uniform(0, width), rng.uniform(0, height), rng.uniform(10, 120)
        field[(x - cx) ** 2 + (y - cy) ** 2 < r * r] = np.float32(cap)
    field[rng.integers(0, height, 6), :] = np.nan
    flat = field.reshape(-1)
    flat[rng.integers(0, flat.size, 500)] = np.inf
    return flat


@pytest.mark.parametrize("fraction", [0.25, 0.5, 0.999, 1.0])
def test_atlas_4k_matches_oracle(product, oracle_port, package, fraction):
    native = package.native
    parent = _structured_field(1920, 1080, 20000, 1)
    child = _structured_field(1920, 1080, 26000, 2)
    args = (parent, (1920, 1080), 20000, child, (1920, 1080), 26000, (3840, 2160), 1.0 / fraction if fraction < 1
            else 1.0, fraction, 30000)
    got = native.atlas_colourise(product, *args, 0.3, 0.4, 0.7, 0.62, interior=(3, 4, 5))
    want = native.atlas_colourise(oracle_port, *args, 0.3, 0.4, 0.7, 0.62, interior=(3, 4, 5))
    np.testing.assert_array_equal(got, want)
    got = native.atlas_field(product, *args, child_zoom=1.25, parent_bias=1.0, child_bias=2.0, output_bias=0.5,
                             feather=48)
    want = native.atlas_field(oracle_port, *args, child_zoom=1.25, parent_bias=1.0, child_bias=2.0, output_bias=0.5,
                              feather=48)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_atlas_errors_match_oracle(product, oracle_port, package):
    native = package.native
    parent = np.zeros(16 * 9, dtype=np.float32)
    messages = []
    for library in (product, oracle_port):
        row = []
        for kwargs in (dict(output_bias=1e9), dict(feather=-1), dict(parent_bias=-1.0)):
            full = dict(child_zoom=1.0, parent_bias=0.0, child_bias=0.0, output_bias=0.0, feather=48)
            full.update(kwargs)
            with pytest.raises(native.NativeError) as error:
                native.atlas_field(library, parent, (16, 9), 100, parent, (16, 9), 100, (16, 9), 1.0, 0.5, 100,
                                   **full)
            row.append(str(error.value).split(": ", 1)[1])
        with pytest.raises(native.NativeError) as error:
            native.atlas_colourise(library, parent, (16, 9), 100, parent, (16, 9), 100, (16, 9), 1.0, 0.5, 100,
                                   0.1, 0.2, 0.3, 0.4, interior=(0, 300, 0))
        row.append(str(error.value).split(": ", 1)[1])
        messages.append(row)
    assert messages[0] == messages[1]
    # The library still works after the failures.
    out = native.atlas_field(product, parent, (16, 9), 100, None, None, 0, (16, 9), 1.0, 0.0, 100)
    assert np.all(out == 0.0)


def test_atlas_device_entries_match_host_entries(product, package):
    """fractal_gb300_atlas_*_device on device buffers equals the host-buffer
    entry points, on the library stream and on a caller stream."""
    import ctypes

    import torch

    native = package.native
    parent = _structured_field(960, 540, 9000, 5)
    child = _structured_field(960, 540, 12000, 6)
    d_parent = torch.from_numpy(parent).cuda()
    d_child = torch.from_numpy(child).cuda()
    width, height = 1920, 1080
    interior = (ctypes.c_int * 3)(7, 8, 9)
    accents = np.asarray(atlas_cases.ACCENTS, dtype=np.uint8)
    for stream in (None, torch.cuda.Stream()):
        handle = stream.cuda_stream if stream is not None else None
        rgb = torch.empty(width * height * 3, dtype=torch.uint8, device="cuda")
        status = product.fractal_gb300_atlas_colourise_device(
            d_parent.data_ptr(), 960, 540, 9000, d_child.data_ptr(), 960, 540, 12000, rgb.data_ptr(), width, height,
            1.6, 0.4, 0, 0.3, 0.4, 0.7, 0.55, interior, accents.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
            handle)
        assert status == 0, native.last_error(product)
        field = torch.empty(width * height, dtype=torch.float32, device="cuda")
        status = product.fractal_gb300_atlas_field_device(
            d_parent.data_ptr(), 960, 540, 9000, d_child.data_ptr(), 960, 540, 12000, field.data_ptr(), width,
            height, 1.6, 0.4, 1.3, 0.5, 0.25, 1.0, 100, 30, handle)
        assert status == 0, native.last_error(product)
        torch.cuda.synchronize()
        want_rgb = native.atlas_colourise(product, parent, (960, 540), 9000, child, (960, 540), 12000,
                                          (width, height), 1.6, 0.4, 0, 0.3, 0.4, 0.7, 0.55, interior=(7, 8, 9),
                                          accents=accents)
        want_field = native.atlas_field(product, parent, (960, 540), 9000, child, (960, 540), 12000,
                                        (width, height), 1.6, 0.4, 100, child_zoom=1.3, parent_bias=0.5,
                                        child_bias=0.25, output_bias=1.0, feather=30)
        np.testing.assert_array_equal(rgb.cpu().numpy(), want_rgb)
        np.testing.assert_array_equal(field.cpu().numpy().view(np.uint32), want_field.view(np.uint32))


def test_kfp_raw_device_matches_host_entry(product, package):
    """fractal_gb300_atlas_colourise_kfp_raw_device (device LUT and fields)
    equals fractal_atlas_colourise_kfp_raw through host buffers."""
    import ctypes

    import torch

    native = package.native
    kfp = package.kfp
    profile = kfp.recipe("seeded16")
    lut = kfp.palette_lut(profile)
    parent = _structured_field(960, 540, 9000, 15)
    child = _structured_field(960, 540, 12000, 16)
    for bias in (0.0, 12000.0):
        p = parent if bias == 0.0 else (parent - np.float32(9000)).astype(np.float32)
        c = child if bias == 0.0 else (child - np.float32(12000)).astype(np.float32)
        options = kfp.options(profile, field_bias=bias)
        want = native.atlas_colourise_kfp_raw(product, p, (960, 540), 9000, c, (960, 540), 12000, (1920, 1080), 1.7,
                                              0.42, 1.0, 12000, options, lut)
        d_p, d_c = torch.from_numpy(p).cuda(), torch.from_numpy(c).cuda()
        d_lut = torch.from_numpy(np.ascontiguousarray(lut)).cuda()
        rgb = torch.empty(1920 * 1080 * 3, dtype=torch.uint8, device="cuda")
        stream = torch.cuda.Stream()
        status = product.fractal_gb300_atlas_colourise_kfp_raw_device(
            d_p.data_ptr(), 960, 540, 9000, d_c.data_ptr(), 960, 540, 12000, rgb.data_ptr(), 1920, 1080, 1.7, 0.42,
            1.0, 12000, ctypes.byref(options), d_lut.data_ptr(), lut.shape[0], stream.cuda_stream)
        assert status == 0, native.last_error(product)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(rgb.cpu().numpy(), want)
