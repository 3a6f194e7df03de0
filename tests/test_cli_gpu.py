"""The EAR command line on the GPU: `calc T60` against the oracle's T60 of
the same rays (through the same FloatBuffer post-processing), `render`
output files, and exact parity on the scene built from the reference's
material presets."""
import json
import os
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from ear_gb300 import Material, Recorder, Source, Tracer, earfile, post

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
CLI = ROOT / "ear_gb300" / "bin" / "EAR"
THREADS = max(1, min(16, os.cpu_count() or 1))


def _scene_from_ear(path):
    sc = earfile.read_ear(path)
    names = [m[0] for m in sc.materials]
    mats = [Material(reflection=m[1], refraction=m[2], specularity=m[3], name=m[0])
            for m in sc.materials]
    v = np.concatenate([t for _, t in sc.meshes], 0)
    ids = np.concatenate([np.full(len(t), names.index(n), np.int32) for n, t in sc.meshes])
    src = Source(location=np.asarray(sc.sources[0]["location"], np.float32),
                 gain=sc.sources[0].get("gain", 1.0))
    recs = [Recorder(location=np.asarray(r["location"], np.float32), channels=r["channels"],
                     right_ear=np.asarray(r.get("right_ear", [1, 0, 0]), np.float32),
                     head_size=r.get("head_size", 0.2),
                     head_absorption=r.get("head_absorption", (0.1, 0.3, 0.9)))
            for r in sc.recorders]
    return sc, v, ids, mats, src, recs


def test_calc_t60_matches_oracle():
    path = GOLDEN / "presets_room.ear"
    r = subprocess.run([str(CLI), "calc", "T60", str(path), "--seed", "11", "--exact"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    vals = dict(re.findall(r"(T60_\w+)\s*:\s*([0-9.]+)s", r.stdout))
    t_ear, t_sab, t_eyr = (float(vals[k]) for k in ("T60_ear", "T60_sabine", "T60_eyring"))
    sc, v, ids, mats, src, recs = _scene_from_ear(path)
    air = sc.settings["absorption"]
    ref = oracle.render(v, ids, mats, src, recs, threads=THREADS, seed=11, context=0, bands=(1,),
                        num_rays=sc.settings["samples"] // 10, max_bounces=999,
                        num_bins=8 * 44100, cutoff=1e-8, air_absorption=air,
                        dry=sc.settings["drylevel"])
    t_ref = post.calc_t60(ref["hist32"][:, 1:2], ref["first_sample"][:, 1:2],
                          ref["last_sample"][:, 1:2], tracks_per_recorder=[1, 2])
    assert t_ear == pytest.approx(t_ref, rel=0.02, abs=2.0 / 44100)
    assert t_sab > 0 and t_eyr > 0


def test_render_writes_impulse_responses(tmp_path):
    path = GOLDEN / "presets_room.ear"
    r = subprocess.run([str(CLI), "render", str(path), "--seed", "3", "--out", str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    wavs = sorted(p.name for p in tmp_path.glob("*.wav"))
    # 2 recorders x 3 bands, reference naming (src/EAR.cpp:234-238)
    assert wavs == sorted(f"response-{i}.sound-0.band-{b}{n}.wav" for i in range(2)
                          for b, n in enumerate(["low", "mid", "high"]))
    head = (tmp_path / "response-1.sound-0.band-1mid.wav").read_bytes()[:44]
    assert head[:4] == b"RIFF" and head[8:16] == b"WAVEfmt " and head[22] == 2  # stereo
    raw = np.fromfile(tmp_path / "response-0.sound-0.band-0low.bin", np.float32)
    assert raw.size > 100 and np.isfinite(raw).all() and np.abs(raw).max() > 0


def test_presets_room_exact_parity():
    sc, v, ids, mats, src, recs = _scene_from_ear(GOLDEN / "presets_room.ear")
    kw = dict(seed=5, context=7, num_rays=3000, max_bounces=999, num_bins=44100 * 2,
              cutoff=1e-8, air_absorption=sc.settings["absorption"], dry=1.0)
    with Tracer(v, ids, mats) as tr:
        res = tr.render(src, recs, exact=True, **kw)
        for band in range(3):
            hit, bt, vis = tr.trace_debug(src, recs, band=band, max_record=120, exact=True, **kw)
            d = oracle.render(v, ids, mats, src, recs, threads=THREADS, debug_band=band,
                              debug_rays=kw["num_rays"], debug_max_record=120,
                              **dict(kw, bands=(band,)))["debug"]
            assert (hit == d[0]).all() and (bt == d[1]).all() and (vis == d[2]).all()
    ref = oracle.render(v, ids, mats, src, recs, threads=THREADS, **kw)
    for key in ("segments", "shadow_queries", "contributions"):
        assert res.stats[key] == ref["counters"][key]
    e1 = (res.hist.astype(np.float64) ** 2).sum(-1)
    e2 = (ref["hist64"] ** 2).sum(-1)
    assert (np.abs(e1 - e2) <= 1e-5 * np.maximum(e2, 1e-300)).all()
