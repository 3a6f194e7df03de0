#!/usr/bin/env python3
"""Benchmark: ray-bounce segments/s of the GB300 ray-tracing core.

A step is one ear_render of the workload: every band of the (source,
keyframe) context, all rays, all recorders -- one pass of the hot path
(Scene::Render, src/Scene.cpp:111-318) over its synthetic scene.  The
default workload is the 2,000,000-triangle cathedral (1 stereo + 8 mono
recorders, 12 materials, 4 s histograms, 300 reflections) at 1e8 rays per
band; the 20,000-triangle relief hall (1e7 rays per band) is reported
beside it in `relief_hall`.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the reference algorithm on the CPU

value      segments/s over the K timed steps, scene resident in HBM, device
           time (CUDA events around each step on its stream; the L2 is
           flushed with a 512 MB write before every step, outside the step).
e2e        the same metric through the C ABI from host memory: scene upload
           from pinned host buffers, BVH and visibility-map builds, render,
           histograms read back to the host, scene release -- all inside
           each timed step.
roofline   algorithmic bytes of the trace kernel (64 B per node visit, 48 B
           per triangle test, 8 B per visibility-map entry, 64 B of path
           state per segment, 4 B per splat bin; counted on the device) /
           its CUDA-event time, against the measured HBM copy bandwidth;
           `l2_frac` against an L2-resident copy measured in the same run.
accuracy   the benchmarked fast kernels against the exact kernels (bit-exact
           to the oracle) on the same rays: largest per-band EDC difference
           down to -40 dB and largest relative T60 difference.
adjoint_ratio  ear_render_adjoint time / ear_render time (configs' inverse
           shoebox, 1e6 rays per band).
cpu_baseline  the CPU restatement of the reference algorithm (brute-force
           triangle loops, oracle/), all host threads, on a bounded ray sample.
auralisation  the steps after the impulse responses (band split, FFT and
           direct convolution of 10 tracks x 3 bands, 4 s x 10 s) with their
           CPU legs; --aural-only runs this part alone.

Multi-GPU (torchrun): rays are independent, so rank r renders rays
[r*N, (r+1)*N) of the same random stream (ear_render_params.first_ray) with
no collective in the data path ("weak" scaling); their raw histograms sum to
one render of world*N rays.  Rank 0 prints the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "relief_hall": "relief_hall",
    "shoebox": "shoebox",
    "cathedral": "cathedral",
}


def load_workload(name: str, num_rays: int | None):
    from ear_gb300 import scenes

    w = getattr(scenes, WORKLOADS[name])()
    if num_rays:
        w.render["num_rays"] = int(num_rays)
    return w


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if _cuda() else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def _cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if _cuda() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if _cuda() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_baseline(w, sample_rays: int, threads: int):
    """The CPU restatement of the reference path on a bounded ray sample:
    the three bands run at once (as the reference's per-band contexts do),
    each band's rays split over threads // 3 threads."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle

    kw = dict(w.render)
    kw["num_rays"] = sample_rays
    per_band = max(1, threads // 3)

    def band(b):
        return oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                             threads=per_band, **dict(kw, bands=(b,)))

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=3) as ex:  # ctypes releases the GIL
        rs = list(ex.map(band, range(3)))
    dt = time.perf_counter() - t0
    seg = sum(r["counters"]["segments"] for r in rs)
    cores = min(threads, 3 * per_band)
    return {"value": seg / dt, "unit": "segments/s", "cores": cores, "kind": "port",
            "sample": f"{sample_rays} rays/band x 3 bands of the same workload, bands at once "
                      f"({seg} segments, {dt:.1f} s, brute-force triangle loops)",
            "seconds": dt, "segments": seg}


def run_reference(args):
    rank, world, local = dist_init(args.gpus)
    if rank != 0:
        return 0
    w = load_workload(args.workload, args.rays)
    threads = os.cpu_count() or 1
    sample = args.cpu_rays or _default_cpu_rays(args.workload)
    for _ in range(args.warmup):
        cpu_baseline(w, max(1, sample // 10), threads)
    vals, segs, secs = [], 0, 0.0
    for _ in range(args.steps):
        b = cpu_baseline(w, sample, threads)
        vals.append(b["value"])
        segs += b["segments"]
        secs += b["seconds"]
    v = segs / secs
    line = {
        "impl": "reference", "metric": "ray-bounce segments/s", "value": v, "unit": "segments/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": _config(w, args),
        "run": {"l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": "segments/s", "cores": 3 * max(1, threads // 3),
                         "kind": "port",
                         "sample": f"{sample} rays/band x 3 bands per step of the workload, "
                                   "brute-force O(T) loops as the reference"},
        "e2e": {"value": v, "unit": "segments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _default_cpu_rays(name):
    return {"relief_hall": 4000, "shoebox": 20000, "cathedral": 5}.get(name, 100)


def _config(w, args):
    """The workload, identical in both arms' lines; how each arm ran it
    goes beside it (`run`)."""
    return {"workload": w.name, "triangles": w.num_triangles, "materials": len(w.materials),
            "recorders": len(w.recorders), "tracks": w.num_tracks,
            "rays_per_band": w.render["num_rays"], "bands": 3,
            "max_bounces": w.render["max_bounces"], "histogram_bins": w.render["num_bins"],
            "cutoff": w.render["cutoff"], "parallelism": f"replicas{args.gpus}"}


def adjoint_ratio(device: int, rays: int, steps: int):
    """Time of the path-replay adjoint (ear_render_adjoint, upstream gradient
    resident on the device) over the time of the forward render it
    differentiates (ear_render, exact kernels, histograms to the device), on
    the 8-material inverse-problem shoebox, CUDA events on the same stream."""
    import torch

    from ear_gb300 import Tracer, scenes

    w, _, _ = scenes.inverse_shoebox(num_rays=rays)
    kw = dict(w.render, exact=True)
    dev = torch.device("cuda", device)
    stream = torch.cuda.current_stream(dev)
    out = torch.zeros((w.num_tracks, 3, kw["num_bins"]), dtype=torch.float32, device=dev)
    g = torch.randn((w.num_tracks, 3, kw["num_bins"]), generator=torch.Generator().manual_seed(0))
    g = g.to(dev)
    with Tracer(w.vertices, w.material_ids, w.materials, device=device) as tr:
        fwd = tr.render(w.source, w.recorders, out=out, **kw)
        book = dict(first=fwd.first_sample, last=fwd.last_sample)

        def run(which):
            if which == "fwd":
                r = tr.render(w.source, w.recorders, out=out, **kw)
                return r.stats
            # the raw bookkeeping comes from a host render of the same rays
            return tr.render_adjoint(w.source, w.recorders, g, raw_first=rf, raw_last=rl, **book,
                                     **kw)[1]

        host = tr.render(w.source, w.recorders, **kw)
        rf, rl = host.raw_first_sample, host.raw_last_sample
        res = {}
        for which in ("fwd", "adj"):
            for _ in range(3):
                run(which)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            seg = 0
            for _ in range(steps):
                seg += int(run(which)["segments"])
            e1.record(stream)
            e1.synchronize()
            res[which] = (e0.elapsed_time(e1) / steps, seg // steps)
    return {"workload": w.name, "rays_per_band": rays, "materials": len(w.materials),
            "forward_ms": res["fwd"][0], "adjoint_ms": res["adj"][0],
            "ratio": res["adj"][0] / res["fwd"][0], "segments_per_pass": res["fwd"][1],
            "adjoint_segments_per_pass": res["adj"][1],
            "path": "ear_render (exact) vs ear_render_adjoint (exact, d_hist on device)"}


def batched_sweep(device: int, rays: int, keyframes: int, full_rays: int, tune_cache=None,
                  curve: str = ""):
    """The batched sweep (16 convex rooms of 500..200,000 triangles, 16
    source / listener pairs each, sources on 24-keyframe paths, 2 s mono
    histograms, 3 bands) rendered two ways on the same GPU: the plain
    per-pair loop (one ear_render per pair-frame, histograms to the device)
    and one autotuned batched launch (ear_batch_run, graph replay).  Point
    1: every pair-frame at ``rays`` rays per band.  Point 2: one pair-frame
    per room at ``full_rays`` rays (the configuration's ray count).  The
    crossover `curve`: the 256 source/listener pairs at keyframe 0, at each
    listed ray count, plus point 2."""
    import torch

    from ear_gb300 import Tracer, scenes
    from ear_gb300.batch import Batch, Job

    rooms, render = scenes.sweep_rooms(keyframes=24)
    kw = {k: v for k, v in render.items() if k != "num_rays"}
    dev = torch.device("cuda", device)
    stream = torch.cuda.current_stream(dev)
    tracers = [Tracer(r.vertices, r.material_ids, r.materials, device=device) for r in rooms]

    def jobs_for(nrays, kf_list, pairs=None):
        jobs = []
        for ri, r in enumerate(rooms):
            for pi in range(len(r.sources) if pairs is None else pairs):
                for k in kf_list:
                    jobs.append(Job(scene=ri, source=r.sources[pi], recorders=[r.listeners[pi]],
                                    keyframe=k, num_rays=nrays, context=(ri * 16 + pi) * 24 + k))
        return jobs

    out = torch.zeros((1, 3, render["num_bins"]), dtype=torch.float32, device=dev)

    def plain(jobs):
        seg = 0
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for j in jobs:
            r = tracers[j.scene].render(j.source, j.recorders, keyframe=j.keyframe, out=out,
                                        **dict(kw, num_rays=j.num_rays, context=j.context))
            seg += int(r.stats["segments"])
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), seg

    def batched(jobs, tune):
        b = Batch(tracers, jobs, stream=stream.cuda_stream, **kw)
        t = None
        if tune:
            t0 = time.perf_counter()
            t = b.tune(trial_fraction=0.05, min_trial_rays=64, tune_leaf_size=True, repeats=1,
                       cache_path=tune_cache, tune_width=True)
            t["tune_s"] = time.perf_counter() - t0
        b.run()  # capture + first replay
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = b.run()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        cfg = b.config
        b.close()
        return ms, int(st["segments"]), cfg, t

    res = {"workload": "sweep: 16 convex rooms (500..200,000 triangles, log-uniform), "
                       "16 source/listener pairs each, 24-keyframe source paths, 2 s mono, 3 bands",
           "triangles": [r.num_triangles for r in rooms]}
    jobs = jobs_for(rays, list(range(keyframes)))
    bms, bseg, cfg, tune = batched(jobs, True)
    pms, pseg = plain(jobs)
    res["all_pair_frames"] = {
        "pair_frames": len(jobs), "rays_per_pair_frame": rays, "keyframes": keyframes,
        "plain_ms": pms, "batched_ms": bms, "speedup": pms / bms,
        "plain_segments_per_s": pseg / (pms / 1000.0), "batched_segments_per_s": bseg / (bms / 1000.0),
        "segments_equal": pseg == bseg, "schedule": cfg, "tuner": tune}
    if full_rays:
        jobs = jobs_for(full_rays, [0], pairs=1)
        bms, bseg, cfg, _ = batched(jobs, False)
        pms, pseg = plain(jobs)
        res["config_rays"] = {
            "pair_frames": len(jobs), "rays_per_pair_frame": full_rays, "plain_ms": pms,
            "batched_ms": bms, "speedup": pms / bms,
            "plain_segments_per_s": pseg / (pms / 1000.0),
            "batched_segments_per_s": bseg / (bms / 1000.0), "segments_equal": pseg == bseg}
    pts = [int(x) for x in curve.split(",") if x.strip()] if curve else []
    if pts:
        res["curve"] = []
        for nr in pts:
            jobs = jobs_for(nr, [0])
            bms, bseg, cfg, _ = batched(jobs, False)
            pms, pseg = plain(jobs)
            res["curve"].append({"pair_frames": len(jobs), "rays_per_pair_frame": nr,
                                 "plain_ms": pms, "batched_ms": bms, "speedup": pms / bms,
                                 "segments_equal": pseg == bseg})
        if "config_rays" in res:
            c = res["config_rays"]
            res["curve"].append({k: c[k] for k in ("pair_frames", "rays_per_pair_frame",
                                                   "plain_ms", "batched_ms", "speedup",
                                                   "segments_equal")})
    for t in tracers:
        t.close()
    return res


def auralisation(device: int, steps: int, cpu: bool):
    """The auralisation after the impulse responses (src/EAR.cpp:295-386) at
    the 10-track shape: 10 recorder tracks x 3 bands of 4 s responses
    (176,400 samples) convolved with 10 s band sections, all 30 contexts in
    one ear_convolve_tracks call, as `EAR render` issues them; plus the band split
    of the 10 s dry sound.  Inputs resident on the device (CUDA events on the
    stream); `e2e` repeats the FFT mode through host buffers.  The CPU legs
    time numpy's FFT convolution per context (the FFTW build's work, one
    thread), the oracle's direct loop nest on a 0.05 s slice (scaled by the
    term count) and the oracle's sequential band split."""
    import torch

    from ear_gb300 import aural
    from ear_gb300.aural import Context, Track

    rng = np.random.default_rng(123)
    dev = torch.device("cuda", device)
    stream = torch.cuda.current_stream(dev)
    n_ir, n_dry, tracks = 176400, 441000, 10
    k = np.arange(n_ir)

    def response(first):
        d = np.zeros(n_ir, np.float32)
        d[first:] = (rng.random(n_ir - first) * np.exp(-(k[first:] - first) / 40000.0)).astype(np.float32)
        return Track(d, first, n_ir - 7)

    dry = (rng.standard_normal(n_dry) * 0.2).astype(np.float32)
    host_ctx = [[Context(response(100 + 31 * t + 7 * b), dry, 0) for b in range(3)]
                for t in range(tracks)]
    dev_dry = torch.from_numpy(dry).to(dev)
    dev_ctx = [[Context(Track(torch.from_numpy(c.ir.data).to(dev), c.ir.first, c.ir.length),
                        dev_dry, 0) for c in row] for row in host_ctx]

    def timed(fn, n):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            r = fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / n, r

    res = {"workload": "10 tracks x 3 bands: 4 s responses (176,400 samples) x 10 s sections "
                       "(441,000 samples); one ear_convolve_tracks call for all tracks"}
    cap = {m: max(aural.processed_capacity(c, m) for c in host_ctx[0]) for m in ("fft", "direct")}
    outs = {m: [torch.zeros(cap[m], device=dev) for _ in range(tracks)] for m in cap}
    kstat = {}

    flat = [c for row in dev_ctx for c in row]
    track_of = [t for t in range(tracks) for _ in range(3)]

    def run(mode):
        for o in outs[mode]:
            o.zero_()
        _, st = aural.convolve_tracks(flat, track_of, mode, outs=outs[mode])
        kstat[mode] = (st["kernel_ms"], st)
        return st["kernel_ms"]

    n = max(1, min(steps, 5))
    fft_ms, _ = timed(lambda: run("fft"), n)
    ks, st = kstat["fft"]
    nctx = 3 * tracks
    npair = (nctx + 1) // 2  # two contexts share one inverse transform
    l = st["fft_points"] // (nctx + npair)  # one transform size for all
    npass = (int(l).bit_length() - 1 + 3) // 4
    # algorithmic bytes of the call: 16 B per point per radix pass over the
    # forward and inverse transforms, 8 B written per packed point + 8 B of
    # inputs read, the product (2 x 8 B read per slot point, 8 B written per
    # pair point) and the accumulate (8 B per result point + 8 B per output
    # sample)
    per_call = 16.0 * (nctx + npair) * l * npass + (8 + 8) * nctx * l + 16 * nctx * l \
        + 8 * npair * l + 8.0 * nctx * (n_ir + n_dry) + 8.0 * tracks * cap["fft"]
    hbm, src = peaks()
    ach = per_call / (ks / 1000.0) / 1e9
    res["fft"] = {"ms": fft_ms, "kernel_ms": ks, "contexts_per_s": 3 * tracks / (fft_ms / 1000.0),
                  "transform_points": int(l), "passes": npass,
                  "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                               "frac": ach / hbm, "peak_source": src,
                               "note": "45 transforms of 8 MB: partly L2-resident"}}
    dir_ms, _ = timed(lambda: run("direct"), 1)
    ks, st = kstat["direct"]
    macs = float(st["multiply_adds"])  # all 30 contexts of the one call
    # FP32 without contraction: a multiply and an add per term, 128 lanes x
    # 152 SMs at the sampled clock
    res["direct"] = {"ms": dir_ms, "kernel_ms": ks, "terms": macs,
                     "terms_per_s": macs / (ks / 1000.0),
                     "note": "bit-identical to the reference's loop order; 2 FP32 instructions per term"}
    bs_ms, _ = timed(lambda: aural.band_split(dev_dry), n)
    bc_ms, _ = timed(lambda: aural.band_split(dev_dry, chunked=True), n)
    res["band_split"] = {"ms_per_10s": bs_ms, "chunked_ms_per_10s": bc_ms,
                         "note": "sequential: bit-identical; chunked: parallel over 512-sample "
                                 "chunks, FP32-filter accuracy"}
    # e2e: host buffers, copies inside the call
    hflat = [c for row in host_ctx for c in row]
    # warm-up: the arena grows once, the output pages are touched once
    houts, _ = aural.convolve_tracks(hflat, track_of, "fft", out_lengths=[cap["fft"]] * tracks)
    for o in houts:
        o.fill(0.0)
    t0 = time.perf_counter()
    aural.convolve_tracks(hflat, track_of, "fft", outs=houts)
    e2e_ms = (time.perf_counter() - t0) * 1000.0
    res["e2e"] = {"fft_ms": e2e_ms, "h2d_bytes": 4 * (3 * tracks * n_ir + n_dry),
                  "d2h_bytes": 4 * tracks * cap["fft"]}
    if cpu:
        import oracle

        c0 = host_ctx[0][0]

        def best(fn, reps=3):  # the fastest of a few runs, in seconds
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                fn()
                ts.append(time.perf_counter() - t0)
            return min(ts)

        m = n_ir - 7 + n_dry + 1

        def fft_ctx():
            a = np.fft.rfft(c0.ir.data[:n_ir - 7].astype(np.float64), m)
            b = np.fft.rfft(dry.astype(np.float64), m)
            np.fft.irfft(a * b, m)

        per_ctx = best(fft_ctx) * 1000.0
        sl = 2205  # 0.05 s
        sc = Context(c0.ir, dry[:sl], 0)
        cap_sl = aural.processed_capacity(sc, "direct")
        oracle.process_direct(Context(c0.ir, dry[:8], 0), 200000)  # loads the library
        dt = best(lambda: oracle.process_direct(sc, cap_sl))
        rate = sl * (c0.ir.length - c0.ir.first) / dt
        bs_cpu = best(lambda: oracle.band_split(dry)) * 1000.0
        res["cpu"] = {"fft_ms_per_context": per_ctx, "fft_ms": per_ctx * 3 * tracks,
                      "direct_terms_per_s": rate, "direct_ms": macs / rate * 1000.0,
                      "band_split_ms_per_10s": bs_cpu, "cores": 1,
                      "kind": "port (numpy FFT; oracle loops)", "timing": "best of 3"}
        res["speedup_fft"] = res["cpu"]["fft_ms"] / fft_ms
        res["speedup_direct"] = res["cpu"]["direct_ms"] / dir_ms
    return res


# DRAM traffic of the trace kernel per launch (dram__bytes_read.sum +
# dram__bytes_write.sum) from ncu captures of the fast kernels with the
# automatic visibility maps, keyed by (workload, rays per band); other
# settings report null.  The cathedral figure is a capture at 1e6 rays per
# band (256.9 GB for 9.979e7 segments) scaled to the 1e8-ray launch by the
# segments rendered (9.978e9): the traffic of a persistent launch grows
# with the paths it traces.
TRAFFIC_PER_LAUNCH = {
    ("relief-hall-20k-stereo", 10_000_000): 16_081_281_024,
    ("cathedral-2M-stereo+8mono", 100_000_000): 25_685_502_702_342,
}


def l2_copy_gbs(dev, mbytes: int = 40, copies: int = 200) -> float:
    """Bandwidth of device-to-device copies whose source and destination
    (2 x mbytes) stay resident in the 126 MB L2: `copies` back-to-back
    copies replayed from one CUDA graph (no launch gaps from the host),
    read + write bytes over the CUDA-event time, best of 5 replays."""
    import torch

    n = mbytes * 1024 * 1024 // 4
    a = torch.ones(n, dtype=torch.float32, device=dev)
    b = torch.empty_like(a)
    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for _ in range(3):
            b.copy_(a)
    torch.cuda.current_stream(dev).wait_stream(side)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(copies):
            b.copy_(a)
    stream = torch.cuda.current_stream(dev)
    g.replay()
    torch.cuda.synchronize(dev)
    best = float("inf")
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.replay()
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n * 4 * copies / (best / 1000.0) / 1e9


def alg_bytes(agg) -> float:
    """Algorithmic bytes of the trace kernel: 64 B per node visit, 48 B per
    triangle test, 64 B of path state per segment, 4 B per splat bin, 8 B
    per visibility-map entry."""
    return 64.0 * agg["node_visits"] + 48.0 * agg["triangle_tests"] + 64.0 * agg["segments"] \
        + 4.0 * agg["splat_bins"] + 8.0 * agg["map_entries"]


AGG_KEYS = ("node_visits", "triangle_tests", "splat_bins", "segments", "rays", "shadow_queries",
            "map_entries")


def timed_renders(tracer, w, kw, out, flush, stream, steps, warmup, exact, world):
    """W warm-up and K timed renders of one workload; CUDA events around
    each step on its stream, L2 flushed before each step (outside it)."""
    import torch

    def step():
        return tracer.render(w.source, w.recorders, out=out, exact=exact, **kw)

    map_build_ms = 0.0
    for _ in range(max(3, warmup)):
        map_build_ms += float(step().stats["map_build_ms"])
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    total_ms = kern_ms = 0.0
    agg = {k: 0 for k in AGG_KEYS}
    res = None
    for _ in range(steps):
        flush.fill_(1.0)
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        res = step()
        s1.record(stream)
        s1.synchronize()
        total_ms += s0.elapsed_time(s1)
        kern_ms += res.stats["kernel_ms"]
        for k in agg:
            agg[k] += int(res.stats[k])
    torch.cuda.synchronize()
    barrier(world)
    return {"total_ms": total_ms, "kernel_ms": kern_ms, "agg": agg, "last": res,
            "map_build_ms": map_build_ms}


def roofline_of(t, steps, hbm, src, l2, traffic):
    ab = alg_bytes(t["agg"])
    ach = ab / (t["kernel_ms"] / 1000.0) / 1e9 if t["kernel_ms"] > 0 else 0.0
    return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "traffic": traffic, "peak_source": src, "kernel": "fast::trace_kernel<0>",
            "algorithmic_bytes_per_launch": ab / steps,
            "kernel_ms_per_launch": t["kernel_ms"] / steps,
            "l2_peak": l2, "l2_frac": ach / l2 if l2 else None,
            "l2_peak_source": "200 graph-replayed device-to-device copies of 40 MB (L2-resident), "
                              "measured in this run"}


def accuracy(local, w, rays):
    """The benchmarked fast kernels against the exact kernels (bit-exact to
    the oracle) on the same rays: post.fast_exact_accuracy."""
    from ear_gb300 import Tracer, post

    kw = dict(w.render, num_rays=int(rays))
    with Tracer(w.vertices, w.material_ids, w.materials, device=local) as tr:
        fast = tr.render(w.source, w.recorders, exact=False, **kw)
        exact = tr.render(w.source, w.recorders, exact=True, **kw)
    acc = post.fast_exact_accuracy(fast, exact)
    acc["rays_per_band"] = int(rays)
    acc["within_target"] = bool(acc["edc_max_db"] < 0.5 and acc["t60_rel"] < 0.02)
    return acc


def run_ours(args):
    import torch

    from ear_gb300 import Tracer

    rank, world, local = dist_init(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.aural_only:  # the auralisation leg alone (profiling its kernels)
        aur = auralisation(local, args.steps, cpu=not args.no_cpu)
        if rank == 0:
            print(json.dumps({"auralisation": aur}))
        return 0
    w = load_workload(args.workload, args.rays)
    kw = dict(w.render)
    # rank r traces rays [r*N, (r+1)*N) of the same random stream: the
    # ranks' raw histograms sum to one render of world*N rays
    kw["first_ray"] = rank * int(kw["num_rays"])
    exact = args.exact
    tracer = Tracer(w.vertices, w.material_ids, w.materials, device=local, box_pad=args.box_pad,
                    builder=args.builder, width=args.width, visibility_map=args.vismap)
    tracks = w.num_tracks
    out = torch.zeros((tracks, 3, kw["num_bins"]), dtype=torch.float32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    hbm, src = peaks()

    clocks = ClockSampler(local)
    clocks.start()
    t_wall = time.perf_counter()
    t = timed_renders(tracer, w, kw, out, flush, stream, args.steps, args.warmup, exact, world)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    t_max = max_over_ranks(t["total_ms"], world)
    agg = t["agg"]
    seg_all = sum_over_ranks(agg["segments"], world)
    value = seg_all / (t_max / 1000.0)
    # per step: first/last init, the persistent trace kernel, finalize
    launches = 3 * args.steps
    res = t["last"]
    l2 = l2_copy_gbs(dev)
    traffic = None
    if not exact and args.vismap == 0:
        traffic = TRAFFIC_PER_LAUNCH.get((w.name, int(kw["num_rays"])))
    roof = roofline_of(t, args.steps, hbm, src, l2, traffic)
    # the timed scene is released before the end-to-end steps, so their own
    # scene and visibility maps get the device memory a caller's would
    bvh_info = tracer.info()
    bvh_info["sah_cost"] = {"binary": tracer.sah_cost(2), "wide4": tracer.sah_cost(4)}
    tracer.close()

    # e2e through the C ABI from pinned host memory, every step
    e2e = None
    if not args.no_e2e:
        vp = torch.from_numpy(np.ascontiguousarray(w.vertices)).pin_memory().numpy()
        mp = torch.from_numpy(np.ascontiguousarray(w.material_ids)).pin_memory().numpy()
        host_out = torch.empty((tracks, 3, kw["num_bins"]), dtype=torch.float32).pin_memory()
        e_steps = max(1, min(args.steps, args.e2e_steps))
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e_seg = 0
        e_map = 0
        e0.record(stream)
        for _ in range(e_steps):
            t2 = Tracer(vp, mp, w.materials, device=local, box_pad=args.box_pad,
                        builder=args.builder, width=args.width, visibility_map=args.vismap)
            r2 = t2.render(w.source, w.recorders, out=host_out, exact=exact, **kw)
            t2.close()
            e_seg += int(r2.stats["segments"])
            e_map = int(r2.stats["map_res"])
        e1.record(stream)
        e1.synchronize()
        e_ms = max_over_ranks(e0.elapsed_time(e1), world)
        e_seg_all = sum_over_ranks(e_seg, world)
        e2e = {"value": e_seg_all / (e_ms / 1000.0), "unit": "segments/s",
               "h2d_bytes_per_step": int(w.vertices.nbytes + w.material_ids.nbytes),
               "d2h_bytes_per_step": int(host_out.numel() * 4),
               "steps": e_steps, "ms_per_step": e_ms / e_steps,
               "visibility_map_cells_per_face_edge": e_map,
               "path": "ear_scene_create (pinned host) + ear_scene_build_bvh + ear_render "
                       "(histograms to pinned host; visibility maps built inside) + "
                       "ear_scene_destroy"}

    # the relief hall (configs' 20,000-triangle scene) beside the headline
    relief = None
    if not args.no_relief and args.workload != "relief_hall":
        wr = load_workload("relief_hall", None)
        kr = dict(wr.render, first_ray=rank * int(wr.render["num_rays"]))
        with Tracer(wr.vertices, wr.material_ids, wr.materials, device=local) as trr:
            outr = torch.zeros((wr.num_tracks, 3, kr["num_bins"]), dtype=torch.float32, device=dev)
            rs = max(1, min(args.steps, 5))
            tr_ = timed_renders(trr, wr, kr, outr, flush, stream, rs, 3, False, world)
        rmax = max_over_ranks(tr_["total_ms"], world)
        relief = {"config": _config(wr, args), "steps": rs,
                  "value": sum_over_ranks(tr_["agg"]["segments"], world) / (rmax / 1000.0),
                  "unit": "segments/s", "ms_per_step": rmax / rs,
                  "rays_per_s": tr_["agg"]["rays"] / (tr_["total_ms"] / 1000.0) * world,
                  "roofline": roofline_of(tr_, rs, hbm, src, l2,
                                          TRAFFIC_PER_LAUNCH.get((wr.name, int(kr["num_rays"])))),
                  "entries_read_per_segment":
                      tr_["agg"]["map_entries"] / max(1, tr_["agg"]["segments"]),
                  "per_segment": {k: tr_["agg"][k] / max(1, tr_["agg"]["segments"])
                                  for k in ("node_visits", "triangle_tests", "splat_bins",
                                            "map_entries")},
                  "gpu_launches": 3 * rs}

    acc = None
    if not args.no_accuracy:
        acc = {w.name: accuracy(local, w, args.accuracy_rays)}
        if args.workload != "relief_hall":
            acc["relief-hall-20k-stereo"] = accuracy(local, load_workload("relief_hall", None),
                                                     args.accuracy_rays)

    bat = None
    if not args.no_batch:
        bat = batched_sweep(local, args.batch_rays, args.batch_keyframes, args.batch_full_rays,
                            curve=args.batch_curve)

    adj = None
    if not args.no_adjoint:
        adj = adjoint_ratio(local, args.adjoint_rays, max(1, min(args.steps, 5)))

    aur = None
    if not args.no_aural:
        aur = auralisation(local, args.steps, cpu=(rank == 0 and world == 1 and not args.no_cpu))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sample = args.cpu_rays or _default_cpu_rays(args.workload)
        cpu = cpu_baseline(w, sample, os.cpu_count() or 1)
        cpu.pop("seconds", None)
        cpu.pop("segments", None)
        # the reference's own threading: one thread per (source, keyframe,
        # band) context (src/EAR.cpp:193-207), i.e. 3 for one context
        ref3 = cpu_baseline(w, max(1, sample // 2), 3)
        cpu["reference_threading"] = {"value": ref3["value"], "unit": "segments/s",
                                      "threads": 3, "sample_rays_per_band": max(1, sample // 2)}

    if rank == 0:
        run = {"l2": "flushed before every step (512 MB write)",
               "mode": "exact (--fmad=false)" if exact else "fast",
               "bvh": bvh_info,
               "rays_per_s": agg["rays"] / (t["total_ms"] / 1000.0) * world}
        # tree quality beside segments/s (unit node and triangle costs): in
        # bvh_info["sah_cost"]
        # the device-counted units of the algorithmic bytes, per segment
        # (a 4-wide node visit counts two 64-byte halves)
        nseg = max(1, agg["segments"])
        run["per_segment"] = {"node_visits_64B": agg["node_visits"] / nseg,
                              "triangle_tests": agg["triangle_tests"] / nseg,
                              "splat_bins": agg["splat_bins"] / nseg,
                              "map_entries": agg["map_entries"] / nseg,
                              "algorithmic_bytes": alg_bytes(agg) / nseg}
        # listener visibility maps (built during warm-up, reused by the
        # timed steps like the tree; e2e builds them inside every step)
        run["visibility_map"] = {"setting": args.vismap, "build_ms": t["map_build_ms"],
                                 "cells_per_face_edge": int(res.stats["map_res"]),
                                 "bytes": int(res.stats["map_bytes"]),
                                 "entries_read_per_segment":
                                     agg["map_entries"] / max(1, agg["segments"]),
                                 "shadow_queries_per_segment":
                                     agg["shadow_queries"] / max(1, agg["segments"])}
        line = {
            "metric": "ray-bounce segments/s", "value": value, "unit": "segments/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": _config(w, args),
            "adjoint_ratio": adj["ratio"] if adj else None,
            "accuracy": acc,
            "roofline": roof,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clk,
            "run": run,
            "relief_hall": relief,
            "adjoint": adj,
            "batched": bat,
            "auralisation": aur,
            "wall_s": wall,
        }
        print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cathedral", choices=sorted(WORKLOADS))
    ap.add_argument("--rays", type=int, default=None, help="rays per band (default: the config's)")
    ap.add_argument("--cpu-rays", type=int, default=None)
    ap.add_argument("--exact", action="store_true")
    ap.add_argument("--box-pad", type=float, default=-1.0)
    ap.add_argument("--builder", default="default", choices=["default", "lbvh", "ploc"])
    ap.add_argument("--width", type=int, default=0, choices=[0, 2, 4],
                    help="BVH traversal width (0: by scene size)")
    ap.add_argument("--vismap", type=int, default=0,
                    help="listener visibility maps: 0 automatic, -1 off, 8..4096 cells per face edge")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-aural", action="store_true")
    ap.add_argument("--no-relief", action="store_true",
                    help="skip the relief-hall object beside the headline workload")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--accuracy-rays", type=int, default=1_000_000,
                    help="rays per band of the fast-vs-exact accuracy renders")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--batch-curve", default="2000,20000,200000",
                    help="rays per pair-frame of the batched crossover curve (one pair-frame "
                         "per source/listener pair, keyframe 0); empty to skip")
    ap.add_argument("--aural-only", action="store_true",
                    help="run only the auralisation leg and print its object")
    ap.add_argument("--batch-rays", type=int, default=2000,
                    help="rays per band and pair-frame of the batched sweep")
    ap.add_argument("--batch-keyframes", type=int, default=24)
    ap.add_argument("--batch-full-rays", type=int, default=1_000_000)
    ap.add_argument("--adjoint-rays", type=int, default=1_000_000)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
