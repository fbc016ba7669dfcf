"""The song workload's audio side: a seeded synthetic track, its per-frame
controls and the camera's zoom plan.

The reference pipeline analyses a real track (visualizer.py:4538, librosa)
and turns its instrumental loudness and onsets into a logarithmic zoom path
with ``_zoom_plan`` (visualizer.py:6982-7074).  Neither librosa nor a track
is available here, so this module

* synthesises a seeded 180 s stereo float32 track at 44.1 kHz: sine tones
  between 110 and 880 Hz, pink noise, a 120-BPM onset train and a slow
  loudness envelope;
* derives per-video-frame controls from it in plain numpy (this module's
  own analysis, not the reference's): the instrumental loudness as an
  attack/release-smoothed RMS envelope normalised to [0, 1], and an onset
  strength from the positive frame-to-frame rise of the RMS;
* restates ``_zoom_plan``: a velocity quiet_speed + (1 + punch) loudness^2.2
  (+ beat_strength onset^1.35) in log10 zoom, integrated, scaled so the last
  frame lands on the maximum, and folded back into [start, max] at both
  bounds.
"""

from __future__ import annotations

import math

import numpy as np


def synthesize(seconds: float = 180.0, sample_rate: int = 44_100, seed: int = 4242, bpm: float = 120.0):
    """A seeded stereo float32 track of shape (samples, 2) in [-1, 1]."""
    rng = np.random.default_rng(seed)
    n = int(round(seconds * sample_rate))
    t = np.arange(n, dtype=np.float64) / sample_rate
    mono = np.zeros(n, dtype=np.float64)
    # Sine tones between 110 and 880 Hz with seeded amplitudes and phases,
    # each fading in and out on its own slow cycle.
    for _ in range(12):
        frequency = float(np.exp(rng.uniform(math.log(110.0), math.log(880.0))))
        amplitude = float(rng.uniform(0.02, 0.08))
        phase = float(rng.uniform(0.0, 2.0 * math.pi))
        swell = 0.5 + 0.5 * np.sin(2.0 * math.pi * t / float(rng.uniform(8.0, 40.0)) + float(rng.uniform(0, 6.3)))
        mono += amplitude * swell * np.sin(2.0 * math.pi * frequency * t + phase)
    # Pink noise: white noise shaped by 1/sqrt(f) in the frequency domain.
    spectrum = np.fft.rfft(rng.standard_normal(n))
    freqs = np.fft.rfftfreq(n, 1.0 / sample_rate)
    spectrum[1:] /= np.sqrt(freqs[1:])
    spectrum[0] = 0.0
    pink = np.fft.irfft(spectrum, n)
    mono += 0.05 * pink / (np.std(pink) + 1e-12)
    # A 120-BPM onset train: decaying 60 Hz kicks on every beat.
    beat = 60.0 / bpm
    since = np.mod(t, beat)
    mono += 0.35 * np.exp(-since / 0.06) * np.sin(2.0 * math.pi * 60.0 * since)
    # A slow loudness envelope (quiet verses, loud choruses).
    mono *= 0.35 + 0.65 * (0.5 - 0.5 * np.cos(2.0 * math.pi * t / 45.0))
    mono /= max(1e-12, float(np.max(np.abs(mono))))
    stereo = np.stack([mono, np.roll(mono, int(0.0007 * sample_rate))], axis=1)
    return stereo.astype(np.float32)


def frame_controls(audio, sample_rate: int = 44_100, fps: float = 60.0, attack: float = 0.025,
                   release: float = 0.25):
    """Per-video-frame (instrumental loudness, onset strength), both in
    [0, 1]: the RMS of each frame's samples smoothed with one-pole attack and
    release time constants, normalised by its 99th percentile; the onset is
    the positive rise of the raw RMS, normalised the same way."""
    mono = np.asarray(audio, dtype=np.float64)
    if mono.ndim == 2:
        mono = mono.mean(axis=1)
    hop = sample_rate / fps
    frames = int(math.floor(len(mono) / hop))
    edges = np.round(np.arange(frames + 1) * hop).astype(np.int64)
    squares = np.concatenate(([0.0], np.cumsum(mono * mono)))
    rms = np.sqrt(np.maximum(0.0, (squares[edges[1:]] - squares[edges[:-1]]) / np.diff(edges)))
    up = 1.0 - math.exp(-1.0 / (attack * fps))
    down = 1.0 - math.exp(-1.0 / (release * fps))
    smooth = np.empty_like(rms)
    level = 0.0
    for i, value in enumerate(rms):
        level += (up if value > level else down) * (value - level)
        smooth[i] = level
    loudness = np.clip(smooth / max(1e-12, float(np.quantile(smooth, 0.99))), 0.0, 1.0)
    rise = np.maximum(0.0, np.diff(rms, prepend=rms[0]))
    onset = np.clip(rise / max(1e-12, float(np.quantile(rise, 0.99))), 0.0, 1.0)
    return loudness, onset


def zoom_plan(loudness, start_log: float, max_log: float, punch: float = 3.0, quiet_speed: float = -0.04,
              onset=None, beat_strength: float = 0.0):
    """log10 zoom per frame from the loudness (and optional onset) controls,
    as the reference's _zoom_plan (visualizer.py:6982-7074) plans it."""
    envelope = np.clip(np.asarray(loudness, dtype=np.float64), 0.0, 1.0)
    if envelope.ndim != 1 or envelope.size == 0:
        raise ValueError("loudness controls must be a non-empty one-dimensional series")
    if max_log <= start_log:
        return np.full(envelope.shape, float(start_log))
    if envelope.size == 1:
        return np.asarray([float(max_log)])
    span = float(max_log) - float(start_log)
    velocity = quiet_speed + (1.0 + punch) * envelope ** 2.2
    if onset is not None and beat_strength != 0.0:
        velocity = velocity + beat_strength * np.clip(np.asarray(onset, dtype=np.float64), 0.0, 1.0) ** 1.35
    travelled = np.concatenate(([0.0], np.cumsum(velocity[:-1])))
    total = float(np.sum(velocity[:-1]))
    if total <= 1.0e-6:
        # No net forward motion: crawl forward instead of running backwards.
        velocity = velocity - float(np.min(velocity)) + 1.0e-3
        travelled = np.concatenate(([0.0], np.cumsum(velocity[:-1])))
        total = max(float(np.sum(velocity[:-1])), 1.0e-6)
    position = travelled / total * span
    # Fold at both bounds (a reflection with period 2 * span).
    folded = np.mod(position, 2.0 * span)
    return float(start_log) + np.where(folded <= span, folded, 2.0 * span - folded)
