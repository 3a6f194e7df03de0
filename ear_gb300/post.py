"""Post-processing of rendered tracks, as the reference's Render() does after
tracing (src/EAR.cpp:209-262), plus Schroeder energy-decay curves.

The per-track operations call the library's host functions (ear_track_*,
restatements of FloatBuffer / RecorderTrack, src/Recorder.cpp:76-118,
303-340) so the CLI, the Python API and the tests share one implementation.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _native as N


def track_power(track: np.ndarray, first: int, last: int, a: float = 0.67) -> None:
    assert track.dtype == np.float32 and track.flags.c_contiguous
    N.check(N.lib().ear_track_power(track.ctypes.data, int(first), int(last), float(a)))


def track_maximum(track: np.ndarray, first: int, last: int) -> float:
    return float(N.lib().ear_track_maximum(track.ctypes.data, int(first), int(last)))


def track_length(track: np.ndarray, first: int, last: int, tresh: float = -1.0) -> int:
    return int(N.lib().ear_track_length(track.ctypes.data, int(track.shape[-1]), int(first),
                                        int(last), float(tresh)))


def track_t60(track: np.ndarray, first: int, last: int) -> float:
    return float(N.lib().ear_track_t60(track.ctypes.data, int(first), int(last)))


def power_and_truncate(tracks: Sequence[np.ndarray], first: Sequence[int], last: Sequence[int],
                       tracks_per_recorder: Sequence[int], power: float = 0.335):
    """src/EAR.cpp:209-228 for one set of rendered recorders: Power(0.335)
    on every track, global maximum, then each recorder truncated to
    getLength(max / 256).  Tracks are modified in place; returns the new
    real_length of every track."""
    for t, f, l in zip(tracks, first, last):
        track_power(t, f, l, power)
    mx = 0.0
    for t, f, l in zip(tracks, first, last):
        mx = max(mx, track_maximum(t, f, l))
    tresh = float(np.float32(mx) / np.float32(256.0))  # float treshold = max / 256.0f
    new_last = list(last)
    i = 0
    for nt in tracks_per_recorder:
        length = 0
        for j in range(i, i + nt):
            length = max(length, track_length(tracks[j], first[j], last[j], tresh))
        # Recorder::Truncate -> FloatBuffer::Truncate (l == 0 -> 1)
        for j in range(i, i + nt):
            new_last[j] = max(length, 1)
        i += nt
    return new_last


def calc_t60(hist_band: np.ndarray, first: np.ndarray, last: np.ndarray,
             tracks_per_recorder: Optional[Sequence[int]] = None) -> float:
    """The ray-traced T60 of `EAR calc T60` (src/EAR.cpp:250-262): the mid
    band of one context, post-processed, then RecorderTrack::T60 of recorder
    0, track 0.  ``hist_band`` is (tracks, bins) or (tracks, 1, bins)."""
    h = np.asarray(hist_band, np.float32)
    if h.ndim == 3:
        h = h[:, 0]
    first = np.asarray(first).reshape(-1)
    last = np.asarray(last).reshape(-1)
    tracks = [np.ascontiguousarray(h[i].copy()) for i in range(h.shape[0])]
    tpr = list(tracks_per_recorder) if tracks_per_recorder is not None else [1] * len(tracks)
    new_last = power_and_truncate(tracks, [int(x) for x in first], [int(x) for x in last], tpr)
    return track_t60(tracks[0], int(first[0]), int(new_last[0]))


def edc_db(h: np.ndarray, floor_db: float = -300.0) -> np.ndarray:
    """Schroeder energy-decay curve of one track in dB:
    EDC(t) = 10 log10( sum_{tau >= t} |h(tau)| / sum |h| ), accumulated in
    FP64 (the recorded values are signed intensities, src/Scene.cpp:256-258,
    so |h| is the energy)."""
    e = np.abs(np.asarray(h, np.float64))
    tail = np.cumsum(e[::-1])[::-1]
    tot = tail[0] if tail.size else 0.0
    if tot <= 0:
        return np.full(e.shape, floor_db)
    with np.errstate(divide="ignore"):
        d = 10.0 * np.log10(tail / tot)
    return np.maximum(d, floor_db)


def edc_db_torch(h, floor_db: float = -300.0):
    """Differentiable EDC in dB for a (..., bins) tensor (FP64 inside)."""
    import torch

    e = h.abs().to(torch.float64)
    tail = torch.flip(torch.cumsum(torch.flip(e, [-1]), -1), [-1])
    tot = tail[..., :1].clamp_min(1e-300)
    return torch.clamp(10.0 * torch.log10((tail / tot).clamp_min(1e-300)), min=floor_db)


def track_t60_alone(h: np.ndarray, first: int, last: int) -> float:
    """RecorderTrack::T60 of one track after the post-processing of
    `EAR calc T60` (Power(0.335), truncation at max / 256) applied to that
    track alone."""
    t = np.ascontiguousarray(np.asarray(h, np.float32).copy())
    new_last = power_and_truncate([t], [int(first)], [int(last)], [1])
    return track_t60(t, int(first), int(new_last[0]))


def fast_exact_accuracy(fast, exact, floor_db: float = -40.0) -> dict:
    """Agreement of two renders of the same rays (``RenderResult``s with
    host histograms): the largest difference of any track's per-band
    Schroeder EDC down to ``floor_db`` (in the second render), and the
    largest relative T60 difference over tracks and bands."""
    hf, he = np.asarray(fast.hist), np.asarray(exact.hist)
    edc_max, t60_rel, worst = 0.0, 0.0, None
    for t in range(he.shape[0]):
        for b in range(3):
            if not he[t, b].any():
                continue
            ef, ee = edc_db(hf[t, b]), edc_db(he[t, b])
            m = ee > floor_db
            d = float(np.abs(ef[m] - ee[m]).max()) if m.any() else 0.0
            if d > edc_max:
                edc_max, worst = d, (t, b)
            tf = track_t60_alone(hf[t, b], fast.first_sample[t, b], fast.last_sample[t, b])
            te = track_t60_alone(he[t, b], exact.first_sample[t, b], exact.last_sample[t, b])
            if te > 0:
                t60_rel = max(t60_rel, abs(tf - te) / te)
    return {"edc_max_db": edc_max, "t60_rel": t60_rel, "edc_floor_db": floor_db,
            "worst_track_band": worst}
