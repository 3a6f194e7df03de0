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


def write_dry(path, seconds=0.4, seed=0):
    """A 16-bit mono dry sound: noise bursts."""
    rng = np.random.default_rng(seed)
    n = int(seconds * 44100)
    env = (np.sin(np.arange(n) / 44100 * 2 * np.pi * 5) > 0.3).astype(np.float64)
    x = np.clip(rng.standard_normal(n) * 0.25 * env, -0.99, 0.99)
    pcm = (x * 32767).astype("<i2")
    data = pcm.tobytes()
    hdr = b"RIFF" + (36 + len(data)).to_bytes(4, "little") + b"WAVEfmt " + (16).to_bytes(4, "little")
    hdr += (1).to_bytes(2, "little") + (1).to_bytes(2, "little") + (44100).to_bytes(4, "little")
    hdr += (88200).to_bytes(4, "little") + (2).to_bytes(2, "little") + (16).to_bytes(2, "little")
    Path(path).write_bytes(hdr + b"data" + len(data).to_bytes(4, "little") + data)
    return (pcm.astype(np.float32) / np.float32(32768.0)).astype(np.float32)


def read_wav16(path):
    b = Path(path).read_bytes()
    ch = int.from_bytes(b[22:24], "little")
    return np.frombuffer(b[44:], "<i2").reshape(-1, ch), b


def test_render_writes_impulse_responses(tmp_path):
    path = GOLDEN / "presets_room.ear"
    write_dry(tmp_path / "dry.wav")
    r = subprocess.run([str(CLI), "render", str(path), "--seed", "3", "--out", str(tmp_path)],
                       capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout
    for name, ch in (("mono.wav", 1), ("stereo.wav", 2)):  # the OUT files, auralised
        pcm, _ = read_wav16(tmp_path / name)
        assert pcm.shape[1] == ch and pcm.shape[0] > 44100
        peak = np.abs(pcm.astype(np.int64)).max()
        assert 0.79 * 32768 <= peak <= 0.8 * 32768 + 1  # Normalize(0.8), Save without norm
    wavs = sorted(p.name for p in tmp_path.glob("response-*.wav"))
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


def keyed_scene(tmp_path, triple=False):
    """The presets room with two keyframes: the source moves, the recorders
    stay; a 0.4 s dry sound (or, triple, three 0.4 s band WAVs: a 3SRC)."""
    sc = earfile.read_ear(GOLDEN / "presets_room.ear")
    loc = np.asarray(sc.sources[0]["location"], np.float32)
    src = {"file": "dry.wav", "location": np.stack([loc, loc + np.float32([0.8, 0.2, 0.0])]),
           "gain": 1.0}
    if triple:
        src["files"] = ["b0.wav", "b1.wav", "b2.wav"]
    recs = [dict(r) for r in sc.recorders]
    settings = dict(sc.settings, samples=20000)
    blob = earfile.encode(materials=sc.materials, meshes=sc.meshes, sources=[src], recorders=recs,
                          settings=settings, keys=[0.0, 0.2], freq=sc.freq)
    (tmp_path / "keyed.ear").write_bytes(blob)
    if triple:
        return sc, [write_dry(tmp_path / f"b{b}.wav", 0.3 + 0.05 * b, seed=10 + b)
                    for b in range(3)]
    return sc, write_dry(tmp_path / "dry.wav", 0.4, seed=4)


def reconstruct(tmp_path, sc, dry, mode):
    """The auralisation of the reference's Render() (src/EAR.cpp:295-386)
    restated in Python on the oracle's convolution, from the tracks the CLI
    dumped: returns {OUT file: int16 samples}."""
    from ear_gb300.aural import Context, Track, section

    keys = [np.float32(0.0), np.float32(0.2)]
    # 3SRC: the three WAVs are the bands (TripleBandSoundFile::Band)
    bands = dry if isinstance(dry, list) else oracle.band_split(dry, sc.freq)
    ctx = []
    for kf in range(2):
        stem = tmp_path / "dump" / f"context-0-{kf}"
        lines = (stem.with_suffix(".txt")).read_text().split("\n")
        tracks, bins = map(int, lines[0].split())
        fl = np.array([list(map(int, l.split())) for l in lines[1:] if l.strip()])
        hist = np.fromfile(stem.with_suffix(".f32"), np.float32).reshape(tracks, 3, bins)
        ctx.append((hist, fl[:, 0].reshape(tracks, 3), fl[:, 1].reshape(tracks, 3)))
    out = {}
    t0 = 0
    for r in sc.recorders:
        chans = []
        for k in range(r["channels"]):
            t = t0 + k
            items = []
            for kf in range(2):
                for b in range(3):
                    hist, first, last = ctx[kf]
                    ir = Track(hist[t, b], int(first[t, b]), int(last[t, b]))
                    if kf == 0:
                        sec, off = section(bands[b], keys[0], float(keys[1] - keys[0]))
                        nh, nf, nl = ctx[1]
                        nxt = Track(nh[t, b], int(nf[t, b]), int(nl[t, b]))
                    else:
                        sec, off = section(bands[b], keys[1])
                        nxt = None
                    items.append(Context(ir, sec, off, nxt))
            from ear_gb300 import aural
            cap = max(aural.processed_capacity(c, mode) for c in items)
            if mode == "direct":
                total, _ = oracle.convolve_direct(items, cap)
            else:
                total, _ = oracle.convolve_fft64(items, cap)
                total = total.astype(np.float32)
            chans.append(total[:cap - 1])
        mx = max(float(np.abs(c).max()) for c in chans)
        f = np.float32(0.8) / np.float32(mx)
        chans = [(c * f).astype(np.float32) for c in chans]
        n = max(len(c) for c in chans)
        pcm = np.zeros((n, len(chans)), np.int16)
        for i, c in enumerate(chans):
            pcm[:len(c), i] = np.trunc(c.astype(np.float32) * np.float32(32768.0)).astype(np.int16)
        out[r["file"]] = pcm
        t0 += r["channels"]
    return out


def test_render_auralises_keyframes_bit_exact_direct(tmp_path):
    """EAR render --conv direct: the OUT files equal, sample for sample, the
    reference's non-FFTW auralisation of the same tracks (keyframe pairs
    interpolated, the last keyframe plain, Add, Normalize(0.8), Save)."""
    sc, dry = keyed_scene(tmp_path)
    r = subprocess.run([str(CLI), "render", "keyed.ear", "--seed", "9", "--exact", "--seconds", "1",
                        "--conv", "direct", "--dump-tracks", "dump"],
                       capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout
    ref = reconstruct(tmp_path, sc, dry, "direct")
    for name, pcm in ref.items():
        got, _ = read_wav16(tmp_path / name)
        assert got.shape == pcm.shape, name
        np.testing.assert_array_equal(got, pcm)


def test_render_auralises_keyframes_fft(tmp_path):
    """EAR render (FFT, the default): within one LSB of the float64
    evaluation of the FFTW build's arithmetic on the same tracks."""
    sc, dry = keyed_scene(tmp_path)
    r = subprocess.run([str(CLI), "render", "keyed.ear", "--seed", "9", "--seconds", "1",
                        "--dump-tracks", "dump"],
                       capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout
    ref = reconstruct(tmp_path, sc, dry, "fft")
    for name, pcm in ref.items():
        got, _ = read_wav16(tmp_path / name)
        assert got.shape == pcm.shape, name
        assert np.abs(got.astype(np.int32) - pcm.astype(np.int32)).max() <= 1, name


def test_render_auralises_a_triple_band_source_bit_exact(tmp_path):
    """A 3SRC source (one WAV per band, no equalizer; bands of unequal
    length) auralised with --conv direct equals the restatement."""
    sc, bands = keyed_scene(tmp_path, triple=True)
    r = subprocess.run([str(CLI), "render", "keyed.ear", "--seed", "5", "--exact", "--seconds", "1",
                        "--conv", "direct", "--dump-tracks", "dump"],
                       capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout
    ref = reconstruct(tmp_path, sc, bands, "direct")
    for name, pcm in ref.items():
        got, _ = read_wav16(tmp_path / name)
        assert got.shape == pcm.shape, name
        np.testing.assert_array_equal(got, pcm)


def test_render_debugdir_writes_the_references_debug_files(tmp_path):
    """With the 'debugdir' setting the CLI writes the reference's debug
    files (src/EAR.cpp:122-146, 229-240, 362-372): the equalizer bands, the
    impulse responses (.wav, .bin) and each context's processed recorder,
    normalised as Recorder::Save(fn) does (mono: peak 0.8 of full scale)."""
    sc = earfile.read_ear(GOLDEN / "presets_room.ear")
    loc = np.asarray(sc.sources[0]["location"], np.float32)
    src = {"file": "dry.wav", "location": np.stack([loc, loc + np.float32([0.5, 0.0, 0.0])])}
    settings = dict(sc.settings, samples=20000, debugdir="dbg")
    blob = earfile.encode(materials=sc.materials, meshes=sc.meshes, sources=[src],
                          recorders=[dict(r) for r in sc.recorders], settings=settings,
                          keys=[0.0, 0.2], freq=sc.freq)
    (tmp_path / "dbg.ear").write_bytes(blob)
    write_dry(tmp_path / "dry.wav", 0.4, seed=2)
    r = subprocess.run([str(CLI), "render", "dbg.ear", "--seed", "2", "--seconds", "1"],
                       capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stdout
    d = tmp_path / "dbg"
    names = {p.name for p in d.iterdir()}
    lomihi = ["low", "mid", "high"]
    for b in range(3):
        assert f"sound-0.band-{b}{lomihi[b]}.wav" in names
        for kf in range(2):
            for ri in range(2):
                assert f"response-{ri}.sound-0.frame-{kf:02d}.band-{b}{lomihi[b]}.wav" in names
                assert f"response-{ri}.sound-0.frame-{kf:02d}.band-{b}{lomihi[b]}.bin" in names
                assert f"rec-{ri}.sound-0.frame-{kf:02d}.band-{b}.wav" in names
    pcm, _ = read_wav16(d / "rec-0.sound-0.frame-00.band-1.wav")
    assert pcm.shape[1] == 1
    assert abs(int(np.abs(pcm.astype(np.int64)).max()) - 0.8 * 32768) <= 2
