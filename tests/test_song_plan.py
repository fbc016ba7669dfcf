"""CPU: the song workload's audio side (song.py).

* zoom_plan equals the reference's own _zoom_plan (visualizer.py:6982-7074)
  on seeded loudness / onset series, punches and speeds (the reference is
  imported read-only where its checkout exists; skipped elsewhere);
* the synthetic track is seeded, stereo float32 in [-1, 1], 180 s at 44.1 kHz
  by default, and its per-frame controls lie in [0, 1] with a beat every
  half second (120 BPM);
* the plan of the synthetic song starts at 1e0, ends at 1e100 and stays
  within them.
"""

from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from .conftest import REFERENCE_SOURCES, load_package


@pytest.fixture(scope="module")
def song():
    return load_package().song


def test_zoom_plan_matches_reference(song):
    if not os.path.isfile(os.path.join(REFERENCE_SOURCES, "visualizer.py")):
        pytest.skip("reference sources are not present on this machine")
    sys.path.insert(0, REFERENCE_SOURCES)
    try:
        import visualizer  # noqa: PLC0415  (reference pipeline, read-only)
    finally:
        sys.path.remove(REFERENCE_SOURCES)
    rng = np.random.default_rng(21)
    for _ in range(60):
        n = int(rng.integers(2, 4000))
        loud = rng.uniform(-0.2, 1.2, n) * (rng.random() < 0.9)
        onset = rng.uniform(0.0, 1.0, n)
        punch = float(rng.choice([0.0, 1.0, 3.0, 7.5]))
        quiet = float(rng.choice([-0.04, -0.5, 0.0, 0.2]))
        beat = float(rng.choice([0.0, 0.0, 0.8, 2.0]))
        top = float(rng.uniform(1.0, 300.0))
        want = visualizer._zoom_plan(loud, 1.0, 10.0 ** min(top, 300.0), punch, quiet, onset, beat)
        got = song.zoom_plan(loud, 0.0, min(top, 300.0), punch, quiet, onset, beat)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-9)


def test_zoom_plan_edge_cases_match_reference(song):
    """A single frame, no zoom range, silence (no net motion: the crawl
    forward) and two silent frames, against the reference's own plan."""
    if not os.path.isfile(os.path.join(REFERENCE_SOURCES, "visualizer.py")):
        pytest.skip("reference sources are not present on this machine")
    sys.path.insert(0, REFERENCE_SOURCES)
    try:
        import visualizer  # noqa: PLC0415  (reference pipeline, read-only)
    finally:
        sys.path.remove(REFERENCE_SOURCES)
    cases = ((np.array([0.5]), 10.0), (np.array([0.2, 0.4, 0.9]), 0.0), (np.zeros(5), 5.0),
             (np.zeros(2), 3.0), (np.full(7, 0.01), 40.0))
    for loud, top in cases:
        want = visualizer._zoom_plan(loud, 1.0, 10.0 ** top, 3.0, -0.04, None, 0.0)
        got = song.zoom_plan(loud, 0.0, top, 3.0, -0.04, None, 0.0)
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-9)
    with pytest.raises(ValueError):
        song.zoom_plan(np.zeros(0), 0.0, 10.0)


def test_synthetic_song_and_controls(song):
    audio = song.synthesize(seconds=6.0)
    assert audio.shape == (6 * 44_100, 2) and audio.dtype == np.float32
    assert np.max(np.abs(audio)) <= 1.0
    np.testing.assert_array_equal(audio, song.synthesize(seconds=6.0))
    loud, onset = song.frame_controls(audio, fps=60.0)
    assert loud.shape == onset.shape == (360,)
    assert loud.min() >= 0.0 and loud.max() <= 1.0 and onset.min() >= 0.0 and onset.max() <= 1.0
    peaks = np.nonzero(onset > 0.5)[0]
    gaps = np.diff(peaks[np.concatenate(([True], np.diff(peaks) > 5))])
    assert np.all(np.abs(gaps - 30) <= 2)  # one beat every 30 frames


def test_song_plan_spans_the_atlas(song):
    loud, onset = song.frame_controls(song.synthesize(seconds=30.0), fps=60.0)
    plan = song.zoom_plan(loud, 0.0, 100.0, 3.0, -0.04, onset, 0.0)
    assert plan[0] == 0.0 and abs(plan[-1] - 100.0) < 1e-9
    assert plan.min() >= 0.0 and plan.max() <= 100.0
