"""GPU: the atlas KFP entries against the reference's stored output.

* fractal_atlas_colourise_kfp: separate parent / child KFP tiles at output
  scale (own stencil edges, own ColorMethod 4 bounds), feather bands of 0, 1,
  small and maximal width, interior blocks in both tiles, a child at the
  corner, filling the frame, or absent;
* fractal_atlas_colourise_kfp_planes: reprojected surface and render planes
  (orbit, iteration + hidden glitches, bailout, DE, phase), centred input, a
  full-frame child, no child, mixed plane sets and a texture.

Every frame is within +-1 per channel of the reference with >= 99.9 % of
bytes exact (the KFP pass computes its transcendentals in FP32).
"""

from __future__ import annotations

import numpy as np
import pytest

from .golden import kfp_atlas_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def atlas_fixture():
    with np.load(kfp_atlas_cases.KFP_ATLAS_FIXTURE) as data:
        return {key: data[key] for key in data.files}


@pytest.mark.parametrize("case", kfp_atlas_cases.kfp_atlas_cases(), ids=lambda c: c["name"])
def test_kfp_atlas_matches_reference_within_one_lsb(product, atlas_fixture, case):
    out = kfp_atlas_cases.run(product, case)
    expected = atlas_fixture[case["name"]]
    assert out.shape == expected.shape
    diff = np.abs(out.astype(np.int16) - expected.astype(np.int16))
    assert diff.max() <= 1, f"max channel difference {diff.max()} at {np.flatnonzero(diff > 1)[:8]}"
    assert np.mean(diff == 0) >= 0.999, f"only {np.mean(diff == 0):.5f} of bytes exact"


def test_kfp_atlas_rejects_bad_child_rectangle(product):
    """A child rectangle that leaves the frame fails with the reference's
    message; the library stays usable."""
    from .golden.runner import _native

    native = _native()
    case = next(c for c in kfp_atlas_cases.kfp_atlas_cases() if c["name"] == "tiles_feather0")
    bad = dict(case, origin=(40, 20))
    with pytest.raises(native.NativeError, match="invalid native KFP atlas child rectangle"):
        kfp_atlas_cases.run(product, bad)
    assert kfp_atlas_cases.run(product, case).shape == (64 * 36 * 3,)
