#!/usr/bin/env python3
"""Benchmark: ray-bounce segments/s of the GB300 ray-tracing core.

A step is one ear_render of the workload: every band of the (source,
keyframe) context, all rays, all recorders -- one pass of the hot path
(Scene::Render, src/Scene.cpp:111-318) over its synthetic scene.  The
default workload is the 20,000-triangle relief hall (stereo recorder, 3 s
histograms, 200 reflections) at 1e7 rays per band.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the reference algorithm on the CPU

value      segments/s over the K timed steps, scene resident in HBM, device
           time (CUDA events around each step on its stream; the L2 is
           flushed with a 512 MB write before every step, outside the step).
e2e        the same metric through the C ABI from host memory: scene upload
           from pinned host buffers, LBVH build, render, histograms read back
           to the host, scene release -- all inside each timed step.
roofline   algorithmic bytes of the trace kernel (64 B per node visit, 48 B
           per triangle test, 64 B of path state per segment, 4 B per splat
           bin; counted on the device) / its CUDA-event time, against the
           measured HBM copy bandwidth.
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
    """The CPU restatement of the reference path on a bounded ray sample."""
    import oracle

    kw = dict(w.render)
    kw["num_rays"] = sample_rays
    t0 = time.perf_counter()
    r = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                      threads=threads, **kw)
    dt = time.perf_counter() - t0
    seg = r["counters"]["segments"]
    return {"value": seg / dt, "unit": "segments/s", "cores": threads, "kind": "port",
            "sample": f"{sample_rays} rays/band x 3 bands of the same workload "
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
        "config": _config(w, args, flush="n/a (CPU)"),
        "cpu_baseline": {"value": v, "unit": "segments/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} rays/band x 3 bands per step of the workload, "
                                   "brute-force O(T) loops as the reference"},
        "e2e": {"value": v, "unit": "segments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _default_cpu_rays(name):
    return {"relief_hall": 4000, "shoebox": 20000, "cathedral": 4}.get(name, 100)


def _config(w, args, flush):
    return {"workload": w.name, "triangles": w.num_triangles, "materials": len(w.materials),
            "recorders": len(w.recorders), "tracks": w.num_tracks,
            "rays_per_band": w.render["num_rays"], "bands": 3,
            "max_bounces": w.render["max_bounces"], "histogram_bins": w.render["num_bins"],
            "cutoff": w.render["cutoff"], "parallelism": f"replicas{args.gpus}",
            "l2": flush}


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


def batched_sweep(device: int, rays: int, keyframes: int, full_rays: int, tune_cache=None):
    """The batched sweep (16 convex rooms of 500..200,000 triangles, 16
    source / listener pairs each, sources on 24-keyframe paths, 2 s mono
    histograms, 3 bands) rendered two ways on the same GPU: the plain
    per-pair loop (one ear_render per pair-frame, histograms to the device)
    and one autotuned batched launch (ear_batch_run, graph replay).  Point
    1: every pair-frame at ``rays`` rays per band.  Point 2: one pair-frame
    per room at ``full_rays`` rays (the configuration's ray count)."""
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


def run_ours(args):
    import ctypes as C

    import torch

    from ear_gb300 import Tracer, _native as N
    from ear_gb300.scene import make_params, recorders_at

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

    def step():
        return tracer.render(w.source, w.recorders, out=out, exact=exact, **kw)

    map_build_ms = 0.0
    for _ in range(max(3, args.warmup)):
        map_build_ms += float(step().stats["map_build_ms"])
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    total_ms = 0.0
    kern_ms = 0.0
    seg = 0
    agg = {"node_visits": 0, "triangle_tests": 0, "splat_bins": 0, "segments": 0, "rays": 0,
           "shadow_queries": 0, "map_entries": 0}
    launches = 0
    t_wall = time.perf_counter()
    for _ in range(args.steps):
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
        # per step: first/last init, the persistent trace kernel, finalize
        launches += 3
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    t_max = max_over_ranks(total_ms, world)
    seg_all = sum_over_ranks(agg["segments"], world)
    value = seg_all / (t_max / 1000.0)

    # roofline of the trace kernel: algorithmic bytes / kernel time
    alg_bytes = 64.0 * agg["node_visits"] + 48.0 * agg["triangle_tests"] + 64.0 * agg["segments"] \
        + 4.0 * agg["splat_bins"] + 8.0 * agg["map_entries"]
    achieved = alg_bytes / (kern_ms / 1000.0) / 1e9 if kern_ms > 0 else 0.0
    hbm, src = peaks()
    per_launch = alg_bytes / args.steps
    # DRAM traffic of the trace kernel per launch, dram__bytes_read.sum +
    # dram__bytes_write.sum from one ncu capture of this default workload
    # (1e7 rays/band, fast kernels, automatic visibility map); other
    # workloads and settings report null
    traffic = None
    if (w.name == "relief-hall-20k-stereo" and int(kw["num_rays"]) == 10_000_000 and not exact
            and args.vismap == 0):
        traffic = 219_903_488

    # e2e through the C ABI from pinned host memory, every step
    e2e = None
    if not args.no_e2e:
        vp = torch.from_numpy(np.ascontiguousarray(w.vertices)).pin_memory().numpy()
        mp = torch.from_numpy(np.ascontiguousarray(w.material_ids)).pin_memory().numpy()
        host_out = torch.empty((tracks, 3, kw["num_bins"]), dtype=torch.float32).pin_memory()
        e_steps = max(1, min(args.steps, 3))
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e_seg = 0
        e0.record(stream)
        for _ in range(e_steps):
            t2 = Tracer(vp, mp, w.materials, device=local, box_pad=args.box_pad,
                        builder=args.builder, width=args.width, visibility_map=args.vismap)
            r2 = t2.render(w.source, w.recorders, out=host_out, exact=exact, **kw)
            t2.close()
            e_seg += int(r2.stats["segments"])
        e1.record(stream)
        e1.synchronize()
        e_ms = max_over_ranks(e0.elapsed_time(e1), world)
        e_seg_all = sum_over_ranks(e_seg, world)
        e2e = {"value": e_seg_all / (e_ms / 1000.0), "unit": "segments/s",
               "h2d_bytes_per_step": int(w.vertices.nbytes + w.material_ids.nbytes),
               "d2h_bytes_per_step": int(host_out.numel() * 4),
               "steps": e_steps, "ms_per_step": e_ms / e_steps,
               "path": "ear_scene_create (pinned host) + ear_scene_build_bvh + ear_render "
                       "(histograms to pinned host) + ear_scene_destroy"}

    bat = None
    if not args.no_batch:
        bat = batched_sweep(local, args.batch_rays, args.batch_keyframes, args.batch_full_rays)

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
        ref3 = cpu_baseline(w, max(1, sample // 4), 3)
        cpu["reference_threading"] = {"value": ref3["value"], "unit": "segments/s",
                                      "threads": 3, "sample_rays_per_band": max(1, sample // 4)}

    if rank == 0:
        cfg = _config(w, args, flush="flushed before every step (512 MB write)")
        cfg["mode"] = "exact (--fmad=false)" if exact else "fast"
        cfg["bvh"] = tracer.info()
        # tree quality beside segments/s (unit node and triangle costs)
        cfg["bvh"]["sah_cost"] = {"binary": tracer.sah_cost(2), "wide4": tracer.sah_cost(4)}
        # listener visibility maps (built during warm-up, reused by the
        # timed steps like the tree; e2e builds them inside every step)
        cfg["visibility_map"] = {"setting": args.vismap, "build_ms": map_build_ms,
                                 "cells_per_face_edge": int(res.stats["map_res"]),
                                 "bytes": int(res.stats["map_bytes"]),
                                 "entries_read_per_segment":
                                     agg["map_entries"] / max(1, agg["segments"]),
                                 "shadow_queries_per_segment":
                                     agg["shadow_queries"] / max(1, agg["segments"])}
        cfg["rays_per_s"] = agg["rays"] / (total_ms / 1000.0) * world
        line = {
            "metric": "ray-bounce segments/s", "value": value, "unit": "segments/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": cfg,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic,
                         "peak_source": src, "kernel": "trace_kernel<false>",
                         "algorithmic_bytes_per_launch": per_launch,
                         "kernel_ms_per_launch": kern_ms / args.steps},
            "e2e": e2e,
            "adjoint": adj,
            "batched": bat,
            "auralisation": aur,
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clk,
            "wall_s": wall,
        }
        print(json.dumps(line))
    tracer.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="relief_hall", choices=sorted(WORKLOADS))
    ap.add_argument("--rays", type=int, default=None, help="rays per band (default: the config's)")
    ap.add_argument("--cpu-rays", type=int, default=None)
    ap.add_argument("--exact", action="store_true")
    ap.add_argument("--box-pad", type=float, default=-1.0)
    ap.add_argument("--builder", default="default", choices=["default", "lbvh", "ploc"])
    ap.add_argument("--width", type=int, default=0, choices=[0, 2, 4],
                    help="BVH traversal width (0: by scene size)")
    ap.add_argument("--vismap", type=int, default=0,
                    help="listener visibility maps: 0 automatic, -1 off, 8..2048 cells per face edge")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-aural", action="store_true")
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
