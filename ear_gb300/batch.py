"""Batched rendering: many (scene, source, recorders) jobs in one launch.

``Batch`` wraps the ``ear_batch_*`` entry points: a sweep over rooms,
source / listener pairs and keyframes is planned once, traced by one
persistent launch that drains a device work queue, and replayed as a CUDA
graph.  ``Batch.tune`` runs the project's autotuner over the launch
schedule (block size, resident blocks per SM, BVH leaf size, tree width).

Every job renders exactly what ``Tracer.render`` renders for the same
scene, source position, recorders, seed and context.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .scene import Recorder, RenderResult, Source, Tracer, make_params


@dataclass
class Job:
    scene: int                      # index into the batch's tracers
    source: Source
    recorders: Sequence[Recorder]
    num_rays: int
    context: int = 0
    keyframe: int = -1              # evaluated for the source and the recorders


class Batch:
    def __init__(self, tracers: Sequence[Tracer], jobs: Sequence[Job], **kw):
        """``kw`` are the shared render settings of ``make_params`` (seed,
        bands, max_bounces, num_bins, cutoff, air_absorption, dry, exact,
        raw, no_direct, stream); rays and context come from each job."""
        if not tracers or not jobs:
            raise ValueError("a batch needs at least one scene and one job")
        self.tracers = list(tracers)
        self.jobs = list(jobs)
        self.params = make_params(**kw)
        self._num_bins = int(self.params.num_bins)
        scenes = (C.c_void_p * len(self.tracers))(*[t._h.value for t in self.tracers])
        cj = (N.EarBatchJob * len(self.jobs))()
        self._keep = []
        self._tracks = []
        for i, j in enumerate(self.jobs):
            if j.source.is_mesh_source:
                raise ValueError("batches take point sources (render area emitters with Tracer)")
            src, _ = j.source.at(j.keyframe)
            recs = (N.EarRecorder * len(j.recorders))()
            for k, r in enumerate(j.recorders):
                recs[k] = r.at(j.keyframe)
            self._keep.append(recs)
            cj[i].scene = int(j.scene)
            cj[i].num_recorders = len(j.recorders)
            cj[i].recorders = recs
            cj[i].source[:] = list(src.location)
            cj[i].gain = float(src.gain)
            cj[i].num_rays = int(j.num_rays)
            cj[i].context = int(j.context) & 0xFFFFFFFF
            self._tracks.append(sum(r.tracks for r in j.recorders))
        h = C.c_void_p()
        N.check(N.lib().ear_batch_create(scenes, len(self.tracers), cj, len(self.jobs),
                                         C.byref(self.params), C.byref(h)))
        self._h = h

    # ------------------------------------------------------------ schedule
    @property
    def config(self) -> dict:
        c = N.EarBatchConfig()
        N.check(N.lib().ear_batch_get_config(self._h, C.byref(c)))
        return c.as_dict()

    def set_config(self, block: int = 0, blocks_per_sm: int = 0, no_graph: bool = False,
                   bvh_width: int = 0) -> None:
        c = N.EarBatchConfig()
        c.block, c.blocks_per_sm, c.no_graph = int(block), int(blocks_per_sm), int(bool(no_graph))
        c.bvh_width = int(bvh_width)
        N.check(N.lib().ear_batch_set_config(self._h, C.byref(c)))

    def tune(self, trial_fraction: float = 0.02, min_trial_rays: int = 256,
             tune_leaf_size: bool = False, repeats: int = 2,
             cache_path: Optional[str] = None, tune_width: bool = False) -> dict:
        """Autotune the launch schedule on trial launches and apply the
        best; returns the chosen schedule and the trial timings."""
        o = N.EarTuneOpts()
        o.trial_fraction = float(trial_fraction)
        o.min_trial_rays = int(min_trial_rays)
        o.tune_leaf_size = int(bool(tune_leaf_size))
        o.repeats = int(repeats)
        o.cache_path = cache_path.encode() if cache_path else None
        o.tune_width = int(bool(tune_width))
        r = N.EarTuneResult()
        N.check(N.lib().ear_batch_tune(self._h, C.byref(o), C.byref(r)))
        return {"best": r.best.as_dict(), "best_ms": r.best_ms, "default_ms": r.default_ms,
                "candidates": r.candidates, "from_cache": bool(r.from_cache)}

    # ----------------------------------------------------------------- run
    def set_sources(self, positions) -> None:
        """Move every job's point source ([jobs, 3]) without re-planning."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(len(self.jobs), 3)
        N.check(N.lib().ear_batch_set_sources(self._h, pos.ctypes.data))

    def run(self) -> dict:
        st = N.EarRenderStats()
        N.check(N.lib().ear_batch_run(self._h, C.byref(st)))
        return st.as_dict()

    def result(self, job: int, out=None) -> RenderResult:
        """Job ``job``'s (tracks, 3, num_bins) histograms (numpy, or in place
        into a CUDA tensor ``out``) with first / last sample."""
        tracks = self._tracks[job]
        first = np.zeros((tracks, 3), np.int32)
        last = np.zeros((tracks, 3), np.int32)
        h = N.EarHistograms()
        if out is None:
            hist = np.zeros((tracks, 3, self._num_bins), np.float32)
            h.data, h.on_device = hist.ctypes.data, 0
            h.first_sample, h.last_sample = first.ctypes.data, last.ctypes.data
            N.check(N.lib().ear_batch_histograms(self._h, int(job), C.byref(h)))
            return RenderResult(hist, first, last, {})
        import torch
        if tuple(out.shape) != (tracks, 3, self._num_bins) or not out.is_contiguous():
            raise ValueError("out must be a contiguous (tracks, 3, num_bins) tensor")
        fd = torch.empty((tracks, 3), dtype=torch.int32, device=out.device)
        ld = torch.empty_like(fd)
        h.data, h.on_device = out.data_ptr(), 1
        h.first_sample, h.last_sample = fd.data_ptr(), ld.data_ptr()
        N.check(N.lib().ear_batch_histograms(self._h, int(job), C.byref(h)))
        return RenderResult(out, fd.cpu().numpy(), ld.cpu().numpy(), {})

    def device_view(self):
        """(data pointer, row stride in floats, rows, first track per job)."""
        ptr, stride, rows = C.c_void_p(), C.c_int32(), C.c_int64()
        ft = np.zeros(len(self.jobs), np.int32)
        N.check(N.lib().ear_batch_device_view(self._h, C.byref(ptr), C.byref(stride),
                                              C.byref(rows), ft.ctypes.data, len(self.jobs)))
        return ptr.value, stride.value, rows.value, ft

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().ear_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
